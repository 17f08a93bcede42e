// Oracle (test infrastructure only): LMA emission and pair creation
// (nonlinear_compton/*, pair_creation/*), FP64 CPU restatement.
#pragma once
#include "fields.h"

namespace orc {

// plane_wave.rs:251-282 / focused_laser.rs:260-281
int lma_radiate(const Laser& laser, const V4& r, const V4& u, double dt, DrawStream& rng, bool classical,
                bool* emitted, RadiationEvent* ev, uint64_t* rejections);
// plane_wave.rs:284-316 / focused_laser.rs:283-306
int lma_pair_create(const Laser& laser, const V4& r, const V4& ell, const Stokes& pol, double dt, DrawStream& rng,
                    double rate_increase, double* prob, Stokes* pol_new, bool* created, PairEvent* ev,
                    uint64_t* rejections);

}  // namespace orc
