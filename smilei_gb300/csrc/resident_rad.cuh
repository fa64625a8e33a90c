// Monte-Carlo radiation on the resident simulation's particles (shared between
// sim.cu, which owns the particles and the step, and radiation.cu, which owns the
// tables, the network and the Monte-Carlo pass).
#pragma once

#include <cstdint>

#include "smilei_gb300.h"

namespace sg {

// One radiating species of a 2D mixed-form simulation, as the pass sees it: tile
// segments of packed node keys and FP32 offsets, momenta, weights and optical depths,
// the E, B_m field arrays (x-major, ghost width 2), and where its photons go.
struct ResidentRad {
    int N[2], np[2], T[2], nt[2], ntiles;
    double dx[2], dxi[2];
    const float *E[3], *Bm[3];
    const int64_t *seg_start;
    const int *count;
    int64_t nslots;   // buffer slots covered by the segments (last start + last capacity)
    const unsigned *key;
    const float *d[2];
    float *p[3];
    const float *w;
    float *tau;
    double dt, qm2;   // qm2 = charge / mass^2
    uint32_t seed;
    const int64_t *step; // device step counter: the random streams of a step
    double *radiated;    // device tallies
    unsigned long long *emissions;
    // macro-photon store (ph_count null: none; an emission's energy then goes to
    // `radiated`): ph_pos[d * ph_cap + k], ph_mom[c * ph_cap + k], ph_w/chi/tau[k]
    int ph_sampling, ph_max_emissions;
    double ph_threshold;
    int64_t ph_cap;
    unsigned long long *ph_count;
    double *ph_pos, *ph_mom, *ph_w, *ph_chi, *ph_tau;
};

// Enqueues the pass on `stream` (FP32 arithmetic; the table, or the network where
// its validation passed).
int launch_radiate_resident( const sg_rad_tables *tables, const sg_mlp *mlp, const ResidentRad &r,
                             cudaStream_t stream );

} // namespace sg
