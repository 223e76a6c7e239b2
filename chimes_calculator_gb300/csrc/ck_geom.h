#pragma once
#include <string>

#include "ck_common.h"

namespace ck {

// set_hmat (serial_chimes_interface.cpp:85-113): h holds the cell vectors as
// columns (scaled by rep+1), hi its inverse by cofactors.
void set_hmat(const double* ca, const double* cb, const double* cc, double* h, double* hi, int rep);

// Fills the host-computed part of a SysDesc (cells, replication, ghost layers,
// search distance, bin capacity) and the cell volume; checks the box against
// the cutoffs.  c2/c3/c4 are max_cutoff_2B/3B/4B.
Status system_geometry(const double* ca, const double* cb, const double* cc, int n_in, bool small,
                       double c2, double c3, double c4, bool has3, bool has4, SysDesc& d, double& vol,
                       std::string& err);

}  // namespace ck
