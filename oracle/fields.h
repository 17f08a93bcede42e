// Oracle (test infrastructure only): FP64 CPU restatement of ptarmigan's
// four field models and the collision loop.  See physics.h.
#pragma once
#include <cstdint>
#include <vector>

#include "../include/ptarmigan_gb300.h"
#include "physics.h"

namespace orc {

enum Eqn { LORENTZ = 0, LANDAU_LIFSHITZ = 1, MODIFIED_LANDAU_LIFSHITZ = 2 };

struct RadiationEvent {
    V4 k, u_prime;
    Stokes pol;
    double a_eff, chi, absorption;
};

struct PairEvent {
    V4 u_e, u_p;
    double frac, a_eff, chi, absorption;
};

// The Laser enum of field/mod.rs:117-123 with the Field trait of
// field/mod.rs:126-192, one struct with a model switch.
struct Laser {
    ptg_laser_desc d;
    V4 wavevector;   // (2 pi / lambda)(1, 0, 0, 1)
    double duration; // focused models: n_cycles * lambda / c
    double bandwidth;

    explicit Laser(const ptg_laser_desc& desc);
    bool lcfa() const { return d.model == PTG_FAST_PLANE_WAVE || d.model == PTG_FAST_FOCUSED_LASER; }
    double omega() const { return SPEED_OF_LIGHT * wavevector.t; }
    double n_cycles() const;
    double max_timestep() const;
    bool contains(const V4& r) const;
    double ideal_initial_z() const;

    // LCFA field models
    void fields(const V4& r, V3* E, V3* B, double* a) const;
    // LMA field models
    double a_sqd(const V4& r) const;
    V4 grad_a_sqd(const V4& r) const;

    // returns r', u', dt_actual, dwork
    void push(const V4& r, const V4& u, double rqm, double dt, int eqn, V4* r_out, V4* u_out, double* dt_out,
              double* dwork) const;
    // status != 0 means the sample failed (error code)
    int radiate(const V4& r, const V4& u, double dt, DrawStream& rng, bool classical, bool* emitted,
                RadiationEvent* ev, uint64_t* rejections) const;
    int pair_create(const V4& r, const V4& ell, const Stokes& pol, double dt, DrawStream& rng, double rate_increase,
                    double* prob, Stokes* pol_new, bool* created, PairEvent* ev, uint64_t* rejections) const;

   private:
    void ffl_beam(const V4& r, V3* reE, V3* imE, V3* reB, V3* imB) const;
    void ffl_envelope(double phase, double* f, double* df) const;
    void fl_envelope(double phase, double* f, double* df) const;
};

struct OracleParticle {
    int species;
    V4 r, u, r0, u0;
    Stokes pol;
    double weight, payload, parent_chi, interaction_count, work;
    uint64_t id, parent_id, primary, stream;
    int generation, flags, status;
};

struct OracleStats {
    uint64_t lepton_steps = 0, photon_steps = 0, emissions = 0, pair_events = 0, rejections = 0, errors = 0;
    uint64_t created = 0;
};

// main.rs:134-289 for one primary; appends the shower's surviving particles.
void collide(const Laser& laser, const ptg_collide_options& o, const OracleParticle& incident, uint64_t seed,
             uint64_t* current_id, std::vector<OracleParticle>& out, OracleStats& st);

}  // namespace orc
