/*
 * serial_chimes_interface -- source-compatible C++ class of the GB300 ChIMES
 * library (reference: serial_interface/src/serial_chimes_interface.h:93-139).
 *
 * calculate() evaluates one periodic configuration on the GPU: ghost images,
 * cluster lists (identical to the reference's), Chebyshev stage and
 * contraction, force/virial reduction.  Energy and forces are accumulated into
 * the caller's values (the energy sum is then divided by (n_replicates+1)^3);
 * stress[9] is overwritten with the virial over the volume.  With
 * allow_replication (small = true) cells shorter than the 2B cutoff are
 * replicated first and `atmtyps` is extended with the replicas' types, as the
 * reference does.
 */
#ifndef CHIMES_GB300_SERIAL_CHIMES_INTERFACE_H
#define CHIMES_GB300_SERIAL_CHIMES_INTERFACE_H

#include <string>
#include <vector>

#include "chimesFF.h"

class serial_chimes_interface : public chimesFF {
public:
    serial_chimes_interface(bool small = true);
    ~serial_chimes_interface();

    bool allow_replication;

    void init_chimesFF(std::string chimesFF_paramfile, int rank);
    void calculate(std::vector<double>& x_in, std::vector<double>& y_in, std::vector<double>& z_in,
                   std::vector<double>& cella_in, std::vector<double>& cellb_in, std::vector<double>& cellc_in,
                   std::vector<std::string>& atmtyps, double& energy, std::vector<std::vector<double> >& force,
                   std::vector<double>& stress);
};

#endif
