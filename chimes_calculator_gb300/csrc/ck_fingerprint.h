// Cluster fingerprints (the reference's FINGERPRINT build and its histogram
// tool): see ck_fingerprint.cu.
#pragma once
#include <string>

#include "ck_engine.h"

namespace ck {

// Cluster-distance histogram of chimesFF/src/FP/multi_calc_histogram.cpp for
// records of one body order (distances d[n][P] in Angstrom, type indices
// t[n][nbody] of the slot's parameter set): counts[nbin] and the number of
// counted pairs.  same = true compares set 1 with itself (pairs j > i; d2/t2
// unused).  Bins cover [0, maxd) with maxd = 3, sqrt(12)+1, sqrt(24)+1 for 2-,
// 3-, 4-body records.
Status fp_histogram(Engine& eng, int slot, int nbody, long long n1, const double* d1, const int* t1, long long n2,
                    const double* d2, const int* t2, bool same, int nbin, long long* counts, long long* nsamples,
                    std::string& err);

}  // namespace ck
