// Gradients of a trap diagnostic with respect to electrode voltages and the
// magnetic field by a hand-written adjoint of the collisionless PIC step
// (push - gather - deposit - Poisson), with checkpoints every K steps and the
// steps in between recomputed.  No reference counterpart (the reference has no
// derivatives); the forward run is the library's own step.
//
// Loss after N steps, over the live particles of every species:
//   L = w_energy * mean(m vz^2 / 2) [eV] + w_lost * (N0 - N_live) / N0.
// The lost fraction changes only when a particle crosses a wall, so its
// pathwise derivative is zero; the energy term carries the gradient.
#pragma once

#include <string>
#include <vector>

#include "sim.hpp"

namespace mag {

struct AdjointConfig {
    uint64_t nsteps = 0;
    int checkpoint = 100;                  // K
    std::vector<std::string> voltage_keys; // config keys that set electrode voltages (u_segment_3, u_endcap, ...)
    bool grad_b = true;                    // also d L / d(Br, Bt, Bz)
    double w_energy = 1.0, w_lost = 1.0;
};

struct AdjointResult {
    double loss = 0, mean_energy_eV = 0, lost_fraction = 0;
    std::vector<double> grad;  // voltage keys in order, then Br, Bt, Bz when grad_b
    int64_t n0 = 0, n_live = 0;
};

class Adjoint {
public:
    // sim: a fresh simulation (particles loaded, advance_init not yet run); it
    // ends holding the state after nsteps steps.
    static AdjointResult run(Sim& sim, const AdjointConfig& cfg);
};

}  // namespace mag
