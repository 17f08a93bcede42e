// The collision loop (src/main.rs:134-289) as a wave of a persistent
// kernel.  One thread owns one particle at a time and steps it through the
// field until it leaves (Field::contains) or decays; when it is done the
// thread takes the next particle of the wave from a global cursor, so lanes
// stay busy although trajectories differ in length.  Secondaries are
// appended to the shower store with one atomic per warp and form the next
// wave.  Waves alternate leptons -> photons -> leptons ...
#pragma once
#include "ptg_fields.cuh"
#include "ptg_fields32.cuh"
#include "ptg_lcfa.cuh"
#include "ptg_lma.cuh"

namespace ptg {

enum { SP_ELECTRON = 0, SP_POSITRON = 1, SP_PHOTON = 2 };
enum { FLAG_INTERMEDIATE = 1, FLAG_DROP = 2 };
enum { ST_OK = 0, ST_OUT_OF_TABLE = 2, ST_SANITY = 3, ST_REJECTION_CAP = 4, ST_UNSUPPORTED = 9 };
// A queue slot reserved by an append that overflowed the store: published
// so that its consumer can retire it (the batch is rerun with a larger store).
enum { ST_PHANTOM = 100 };

// Shower store, structure of arrays.  Four-vectors are component-major:
// component c of particle i is at v[c * cap + i].
struct Store {
    double *r, *u, *r0, *u0, *pol;
    double *weight, *payload, *parent_chi, *icount, *work;
    unsigned long long *id, *parent_id, *primary, *stream;
    int *species, *generation, *flags, *status;
    int* coll;              // collision of each particle (multi-collision queue)
    unsigned int* ready;    // queue: slot written and published
    unsigned long long cap;
};

struct Counters {
    unsigned long long n_total;  // particles in the store
    unsigned long long next;     // wave cursor
    unsigned long long overflow; // appends that did not fit
    unsigned long long lepton_steps, photon_steps, emissions, pair_events, rejections, errors;
    unsigned long long n_out;    // compaction cursor
    unsigned long long completed; // queue: slots finished (children appended)
    unsigned long long timeouts;  // queue: bounded waits that ran out
    unsigned long long max_steps; // most steps any one particle took
    unsigned long long free_steps; // steps that only drifted (outside the pulse, drifting photons)
    unsigned long long drift_steps; // of those, the drifting photons' steps
};

struct StepOptions {
    double dt;                // max_timestep * dt_multiplier
    double t_stop;            // seconds
    double rate_increase;
    int eqn;                  // EQN_*
    int classical_mode;       // RadiationMode::Classical
    int classical;            // options.classical
    int electron_recoils;
    int tracking_photons;
    int pol_resolved;
    int rotate_stokes;
    int tracking_secondaries;
    int max_generation;       // -1: no limit
    int keep_decayed;
    int has_t_stop;           // t_stop is finite
    uint32_t step_cap;        // steps after which a particle still in the field is retired
    int rej_cap;              // iterations any rejection loop may take
};

struct WaveArgs {
    FieldParams f;
    StepOptions o;
    Store s;
    Counters* c;
    const PairGL* gl;
    const LmaTables* lma;
    double* dbw;                   // DoubleBessel workspaces (LP LMA), one slot per resident lane
    int db_cap;                    // orders per slot
    DbPool dbpool;                 // shared larger slots (pair creation at small eta)
    MlpParams mlp;                 // learned CP proposal (enabled = 0: the reference sampler)
    unsigned long long seed;
    unsigned long long lo, hi;     // wave = store slots [lo, hi)
    unsigned long long n_primaries, id_base;
    // processing order of the wave's slots (offsets from lo), or NULL for
    // slot order; the results do not depend on it (streams are fixed per
    // particle), only how coherently the lanes of a warp step
    const unsigned long long* order;
    // nonzero: each warp takes 32 consecutive particles of that order and
    // the next 32 once all of them are done (warp_load), so that its lanes
    // stay at nearly the same laser phase; zero: each lane takes the next
    // particle as soon as its own is done (lane_load)
    int warp_batch;
};

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// Warp-aggregated append of `count` slots per calling lane (all calling
// lanes must pass the same count).  Returns this lane's first slot.
__device__ __forceinline__ unsigned long long append_slots(Counters* c, unsigned count) {
    unsigned mask = __activemask();
    unsigned leader = __ffs(mask) - 1;
    unsigned rank = __popc(mask & ((1u << lane_id()) - 1u));
    unsigned long long base = 0;
    if (lane_id() == leader) base = atomicAdd(&c->n_total, (unsigned long long)(count * __popc(mask)));
    base = __shfl_sync(mask, base, leader);
    return base + (unsigned long long)rank * count;
}

__device__ __forceinline__ void put4(double* v, unsigned long long cap, unsigned long long i, d4 x) {
    v[i] = x.t;
    v[cap + i] = x.x;
    v[2 * cap + i] = x.y;
    v[3 * cap + i] = x.z;
}
__device__ __forceinline__ d4 get4(const double* v, unsigned long long cap, unsigned long long i) {
    return d4{v[i], v[cap + i], v[2 * cap + i], v[3 * cap + i]};
}

struct Lane {
    d4 r, u, pol;
    double weight, icount, work;
    double hph;  // photons: c dt / ell^0
    double hh;   // leptons: c dt / (2 u^0), the half-drift factor
    unsigned long long slot, stream, id;
    uint32_t step;
    int species, gen, status, flags;
    int coll;
    bool decayed;
    // LMA leptons: the last step was field-free and left u^0 unchanged, so
    // `hh` holds that step's half-drift factor (c/2)(dt / u^0) (lma_drift)
    bool drift_cached;
};

// A field-free LMA lepton step (lma_push_field_free).  Its momentum is
// unchanged and u^0 is recomputed from it, so once a step has left u^0 as
// it found it, every later field-free step reproduces the same u^0, the
// same dt / u^0 and the same half-drift factor: those steps only add h u
// twice, with the same additions, and skip the division and the square
// root.
__device__ __forceinline__ void lma_drift(Lane& L, double dt) {
    if (L.drift_cached) {
        double h = L.hh;
        d4 r = d4{L.r.t + h * L.u.t, L.r.x + h * L.u.x, L.r.y + h * L.u.y, L.r.z + h * L.u.z};
        L.r = d4{r.t + h * L.u.t, r.x + h * L.u.x, r.y + h * L.u.y, r.z + h * L.u.z};
        return;
    }
    double u0t = L.u.t, dt_actual;
    lma_push_field_free(L.r, L.u, dt, &L.r, &L.u, &dt_actual);
    if (L.u.t == u0t) {
        L.drift_cached = true;
        L.hh = 0.5 * SPEED_OF_LIGHT * (dt / L.u.t);
    }
}

__device__ __forceinline__ bool lane_untracked(const WaveArgs& a, const Lane& L) {
    return (!a.o.tracking_secondaries && L.gen > 0) || (a.o.max_generation >= 0 && L.gen > a.o.max_generation);
}

// Default number of steps after which a particle that is still inside the
// field is retired with PTG_ERR_REJECTION_CAP (an iteration cap; the
// context's limits may lower it).  The reference steps until the particle
// leaves the field, which a particle co-moving with the laser (its phase
// k(t - z) advancing by ever less) may never do; every configuration
// measured here stays below 1e6 steps per particle.
constexpr uint32_t STEP_CAP = 1u << 26;

// True when the lane's particle is finished before its next step: failed,
// untracked, or at the step cap (which marks it failed).
__device__ __forceinline__ bool lane_stops(const WaveArgs& a, Lane& L) {
    if (L.status == ST_OK && L.step >= a.o.step_cap) L.status = ST_REJECTION_CAP;
    return L.status != ST_OK || lane_untracked(a, L);
}

// Longest run of field-free steps lma_free_run takes at once.
constexpr uint32_t FREE_RUN_MAX = 4096;

// The field-free LMA lepton steps that follow a field-free step, taken as
// one run.  The phase k(t - z) of a massive particle grows by at most
// 2 omega dt per step and never falls (lma_step_field_free).  So a lepton
// at phase p, before the pulse or after it, stays field-free and inside the
// field (Field::contains: phase < max_phase) for the next m steps, where m
// follows from p alone with a margin of 1 for rounding.  The run then takes
// m steps with lma_drift's own arithmetic and no per-step checks: r, u and
// the step count are bit for bit those of stepping.  Returns m; 0 with a
// t_stop, outside the LMA models, or when the bound leaves no room.
__device__ __forceinline__ uint32_t lma_free_run(const WaveArgs& a, Lane& L) {
    const FieldParams& f = a.f;
    if (!(f.lma_cut > 0.0) || a.o.has_t_stop || L.status != ST_OK) return 0;
    const double dt = a.o.dt;
    const double dphase = 2.0 * f.omega * dt;
    const double phase = phase_of(f, L.r);
    double room = f.max_phase - 1.0 - phase;                          // contains, before every step
    if (!(phase > f.lma_cut + 1.0)) room = fmin(room, -f.lma_cut - 2.0 - phase);  // ends before the pulse
    if (!(dphase > 0.0) || !(room >= dphase)) return 0;
    double mm = floor(room / dphase);
    uint32_t m = mm < (double)FREE_RUN_MAX ? (uint32_t)mm : FREE_RUN_MAX;
    uint32_t left = L.step < a.o.step_cap ? a.o.step_cap - L.step : 0u;  // lane_stops' cap
    m = m < left ? m : left;
    for (uint32_t k = 0; k < m; ++k) lma_drift(L, dt);
    return m;
}

__device__ __forceinline__ void spawn(const WaveArgs& a, unsigned long long slot, int species, d4 r, d4 u, d4 u0,
                                      d4 pol, double weight, double payload, double parent_chi, double work,
                                      unsigned long long parent_id, unsigned long long primary,
                                      unsigned long long stream, int gen) {
    const Store& s = a.s;
    unsigned long long cap = s.cap;
    put4(s.r, cap, slot, r);
    put4(s.r0, cap, slot, r);
    put4(s.u, cap, slot, u);
    put4(s.u0, cap, slot, u0);
    put4(s.pol, cap, slot, pol);
    s.weight[slot] = weight;
    s.payload[slot] = payload;
    s.parent_chi[slot] = parent_chi;
    s.icount[slot] = 0.0;
    s.work[slot] = work;
    s.id[slot] = a.id_base + (slot - a.n_primaries);
    s.parent_id[slot] = parent_id;
    s.primary[slot] = primary;
    s.stream[slot] = stream;
    s.species[slot] = species;
    s.generation[slot] = gen;
    s.flags[slot] = 0;
    s.status[slot] = ST_OK;
}

// Queue mode: a spawned slot is published (collision index, then the ready
// flag with release semantics) after its data is written.
__device__ __forceinline__ void publish_slot(const WaveArgs& a, unsigned long long slot, int coll) {
    a.s.coll[slot] = coll;
    __threadfence();
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(a.s.ready + slot), "r"(1u) : "memory");
}

// Queue mode: slots of an append that did not fit.  Those inside the store
// are published as phantoms; those beyond it are counted as finished here,
// since no consumer will ever read them.
__device__ __forceinline__ void retire_overflow(const WaveArgs& a, unsigned long long slot, unsigned count) {
    for (unsigned q = 0; q < count; ++q) {
        unsigned long long sl = slot + q;
        if (sl < a.s.cap) {
            a.s.status[sl] = ST_PHANTOM;
            publish_slot(a, sl, 0);
        } else {
            atomicAdd(&a.c->completed, 1ull);
        }
    }
}

// One charged-particle step: main.rs:170-206.  Returns true when the step
// only drifted (outside the pulse).
template <int MODEL, bool QUEUE = false>
__device__ __forceinline__ bool lepton_step(const WaveArgs& a, Lane& L, uint32_t* rej, uint32_t* nemit,
                                            LpDefer* dfr = nullptr) {
    const FieldParams& f = a.f;
    double rqm = (L.species == SP_ELECTRON ? ELECTRON_CHARGE : -ELECTRON_CHARGE) / ELECTRON_MASS;
    double dt = a.o.dt;
    d4 r, u;
    double dt_actual, dwork;
    Draws rng;
    rng.begin(a.seed, L.stream, L.step, a.o.rej_cap);
    bool emitted = false;
    d4 k = d4{0, 0, 0, 0}, upr = d4{0, 0, 0, 0};
    d3 kpol = mk3(0, 0, 0);
    double a_eff = 0.0, chi = 0.0, absorption = 0.0;
    bool free_step = false;
    if (MODEL == M_FAST_PLANE_WAVE || MODEL == M_FAST_FOCUSED_LASER) {
        // Field::push default (field/mod.rs:147-152); h = c dt / (2 u^0) was
        // computed by the previous step (or at load)
        double h = L.hh;
        d4 rh = d4{L.r.t + h * L.u.t, L.r.x + h * L.u.x, L.r.y + h * L.u.y, L.r.z + h * L.u.z};
        if (f.env_cut > 0.0 && fabs(phase_of(f, rh)) > f.env_cut) {
            // E = B = 0 at rh: lcf.rs:18-78 then leaves u unchanged bit for
            // bit (every field term is an exact zero), recomputes gamma and
            // drifts the second half step; no work is done.
            u = L.u;
            double g2 = 1.0 + (u.x * u.x + u.y * u.y + u.z * u.z);
            double ig = rsqrt(g2);
            u.t = g2 * ig;  // gamma, as vay_push forms it
            double h2 = (0.5 * SPEED_OF_LIGHT * dt) * ig;
            r = d4{rh.t + h2 * u.t, rh.x + h2 * u.x, rh.y + h2 * u.y, rh.z + h2 * u.z};
            dwork = 0.0;
            L.hh = h2;
            free_step = true;
        } else {
            d3 E, B;
            double aa;
            lcfa_fields(f, rh, &E, &B, &aa);
            vay_push(rh, L.u, E, B, rqm, dt, a.o.eqn, [](double c) { return gaunt_factor(c); }, &r, &u, &dwork, &L.hh);
        }
        dt_actual = dt;
        // lcf.rs:85-134 at the new position.  The per-step probability
        // needs chi only to rate-table precision: FP32 fields and rate.
        float prob = 0.0f;
        {
            f3 e, b;
            if (lcfa_fields32(f, r, &e, &b)) {
                float ig = 1.0f / (float)u.t;
                f3 bt = f3{(float)u.x * ig, (float)u.y * ig, (float)u.z * ig};
                f3 t = f3add(e, f3cross(bt, b));
                float eb = f3dot(e, bt);
                float q = f3dot(t, t) - eb * eb;
                float chi32 = q > 0.0f ? ((float)u.t * f.chi_scale32) * sqrtf(q) : 0.0f;
                float gam = (float)u.t;
                prob = (float)dt_actual * (a.o.classical_mode ? (float)(SQRT_3 * ALPHA_FINE * 5.0 * FRAC_PI_3 / (2.0 * PI * COMPTON_TIME)) * chi32 / gam
                                                             : lcfa_photon_rate32(chi32, gam, a.gl->ln_h32));
            }
        }
        if (prob > 0.0f && rng.next() < (double)prob) {
            // the event: fields, chi and the sample in FP64
            d3 E, B;
            lcfa_fields(f, r, &E, &B, &a_eff);
            d3 beta = mk3(u.x / u.t, u.y / u.t, u.z / u.t);
            double eb = dot(E, beta);
            double E_rf_sqd = norm_sqr(E + SPEED_OF_LIGHT * cross(beta, B)) - eb * eb;
            chi = E_rf_sqd > 0.0 ? u.t * sqrt(E_rf_sqd) / CRITICAL_FIELD : 0.0;
            double r1 = rng.next(), r2 = rng.next(), r3 = rng.next();
            double omega_mc2, theta;
            if (a.o.classical_mode)
                lcfa_classical_sample(chi, u.t, r1, r2, r3, &omega_mc2, &theta);
            else
                lcfa_photon_sample(chi, u.t, r1, r2, r3, &omega_mc2, &theta);
            if (theta >= 0.0 && chi > 0.0) {
                double cphi = 2.0 * PI * r3;
                d3 lng = normalize(beta);
                d3 w = -normalize(E - (dot(lng, E) / sqrt(norm_sqr(E))) * lng + SPEED_OF_LIGHT * cross(beta, B));
                double sp, cp;
                sincos(cphi, &sp, &cp);
                d3 perp = rotate_around(w, lng, sp, cp);
                double st, ct;
                sincos(theta, &st, &ct);
                d3 k3 = omega_mc2 * (ct * lng + st * perp);
                k = d4{sqrt(dot(k3, k3)), k3.x, k3.y, k3.z};
                kpol = lcfa_stokes(k, chi, u.t, beta, w, a.o.classical_mode != 0);
                upr = d4{u.t - k.t, u.x - k.x, u.y - k.y, u.z - k.z};
                emitted = true;
            }
        }
    } else {
        if (lma_step_field_free(f, L.r, dt)) {
            // outside the pulse: the step only drifts, and its emission
            // probability (proportional to <a^2> < 2^-60) is below every
            // nonzero uniform, so it draws nothing
            lma_drift(L, dt);
            return true;
        }
        L.drift_cached = false;
        lma_push(f, L.r, L.u, rqm, dt, a.o.eqn, &r, &u, &dt_actual, &dwork);
        DbWork dbw{nullptr, 0, 32};
        if (a.dbw) {
            size_t warp = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
            dbw.base = a.dbw + warp * (size_t)a.db_cap * 5 * 32 + lane_id();
            dbw.cap = a.db_cap;
            dbw.pool = a.dbpool;
        }
        int st = lma_radiate(f, *a.lma, dbw, a.mlp, r, u, dt_actual, rng, a.o.classical_mode != 0, &emitted, &k, &upr,
                             &kpol, &a_eff, &chi, &absorption, rej, dfr);
        if (st == LMA_DEFERRED) return false;  // the step repeats once the warp has sampled
        if (st != ST_OK) {
            L.status = st;
            L.r = r;
            L.u = u;
            return false;
        }
    }
    if (emitted) {
        unsigned long long slot = append_slots(a.c, 1);
        if (slot < a.s.cap) {
            spawn(a, slot, SP_PHOTON, r, k, d4{0, 0, 0, 0}, d4{1.0, kpol.x, kpol.y, kpol.z}, L.weight, a_eff, chi, 0.0,
                  L.id, a.s.primary[L.slot], child_stream(L.stream, L.step, 0), L.gen + 1);
            if (QUEUE) publish_slot(a, slot, L.coll);
        } else {
            atomicAdd(&a.c->overflow, 1ull);
            if (QUEUE) retire_overflow(a, slot, 1);
        }
        ++*nemit;
        if (a.o.electron_recoils) {
            u = upr;
            L.hh = 0.5 * SPEED_OF_LIGHT * dt / u.t;
        }
        L.icount += 1.0;
        if (!a.o.classical) L.work += absorption;
    }
    L.r = r;
    L.u = u;
    L.work += dwork;
    return free_step;
}

// Steps of a drifting photon taken one by one before the rest of its path
// is found in closed form.
constexpr uint32_t DRIFT_EXACT = 1u << 18;

// True for a photon whose pair probability is zero on every step it has
// left: an LCFA photon below the field's drift threshold, unpolarised as the
// step sees it (pol_resolved off).
__device__ __forceinline__ bool photon_drifts(const WaveArgs& a, const Lane& L) {
    return L.species == SP_PHOTON && !a.o.pol_resolved && L.u.t < a.f.drift_ell_max;
}

// The rest of a drifting photon's path (main.rs:212-264 with a pair
// probability of exactly zero): the step then leaves ell, the weight, the
// Stokes vector and the interaction count as they are and draws nothing, so
// it is r += (c dt / ell^0) ell until the photon leaves the field
// (Field::contains) or reaches t_stop.  The first DRIFT_EXACT steps repeat
// photon_step's additions, so r is bit for bit what stepping gives; a
// photon still inside after them (one moving nearly with the laser, whose
// phase k(t - z) advances by ever less) jumps to a few steps short of its
// exit in closed form, r += (m h) ell, with a relative error of a few
// ulps times the steps it jumps, and takes the last steps one by one.
// Returns the steps taken; a photon whose phase cannot advance is retired
// at the step cap.
static __device__ __noinline__ unsigned long long photon_drift(const WaveArgs& a, Lane& L) {
    const FieldParams& f = a.f;
    const double h = L.hph;
    const d4 ell = L.u;
    d4 r = L.r;
    unsigned long long steps = 0;
    auto inside = [&](const d4& p) {
        return contains(f, p) && (!a.o.has_t_stop || p.t / SPEED_OF_LIGHT < a.o.t_stop);
    };
    for (int jump = 0; jump < 4; ++jump) {
        for (uint32_t k = 0; k < DRIFT_EXACT; ++k) {
            if (!inside(r)) {
                L.r = r;
                return steps;
            }
            r = d4{r.t + h * ell.t, r.x + h * ell.x, r.y + h * ell.y, r.z + h * ell.z};
            ++steps;
        }
        // steps left to the exit: the phase advances by k h (ell^0 - ell_z)
        // per step, the time by h ell^0
        double dphase = f.k * h * (ell.t - ell.z);
        double left = dphase > 0.0 ? (f.max_phase - phase_of(f, r)) / dphase : HUGE_VAL;
        if (a.o.has_t_stop) left = fmin(left, (a.o.t_stop * SPEED_OF_LIGHT - r.t) / (h * ell.t));
        if (!(left < 4503599627370496.0)) break;  // 2^52: the photon cannot leave
        double m = floor(left) - 4.0;
        if (m > 0.0) {
            double hm = h * m;
            r = d4{r.t + hm * ell.t, r.x + hm * ell.x, r.y + hm * ell.y, r.z + hm * ell.z};
            steps += (unsigned long long)m;
        }
    }
    L.r = r;
    L.status = ST_REJECTION_CAP;
    return steps;
}

// One photon step: main.rs:214-256.
template <int MODEL, bool QUEUE = false>
__device__ __forceinline__ void photon_step(const WaveArgs& a, Lane& L, uint32_t* rej, uint32_t* npair,
                                            BwDefer* bdf = nullptr) {
    const FieldParams& f = a.f;
    double dt = a.o.dt;
    Draws rng;
    rng.begin(a.seed, L.stream, L.step, a.o.rej_cap);
    d4 ell = L.u;
    double h = L.hph;  // c dt / ell^0, fixed for a photon
    d4 r = d4{L.r.t + h * ell.t, L.r.x + h * ell.x, L.r.y + h * ell.y, L.r.z + h * ell.z};
    d4 pol = a.o.pol_resolved ? L.pol : d4{1.0, 0.0, 0.0, 0.0};
    double prob = 0.0;
    d4 pol_new = pol;
    bool created = false;
    d4 ue, up;
    double frac = 1.0, a_eff = 0.0, chi = 0.0, absorption = 0.0;
    if (MODEL == M_FAST_PLANE_WAVE || MODEL == M_FAST_FOCUSED_LASER) {
        // lcf.rs:144-193.  Unpolarised photons: the step probability from
        // FP32 fields and T(chi); polarisation-resolved photons take the
        // FP64 path (their Stokes vector is integrated step by step).
        double prob_step = 0.0;
        if (!a.o.pol_resolved) {
            f3 e, b;
            if (lcfa_fields32(f, r, &e, &b)) {
                f3 l3 = f3{(float)ell.x, (float)ell.y, (float)ell.z};
                f3 n = f3scale(rsqrtf(f3dot(l3, l3)), l3);
                f3 ap = f3add(f3add(e, f3scale(-f3dot(e, n), n)), f3cross(n, b));
                float q = f3dot(ap, ap);
                if (q > 0.0f) {
                    float chi32 = ((float)ell.t * f.chi_scale32) * sqrtf(q);
                    prob_step = (double)((float)(ALPHA_FINE / COMPTON_TIME) * ((float)dt / (float)ell.t) * chi32 *
                                         lcfa_t_mean32(chi32, a.gl->ln_t32));
                }
            }
        }
        bool need64 = a.o.pol_resolved;
        double ri = (prob_step * a.o.rate_increase > 0.1) ? 0.1 / prob_step : a.o.rate_increase;
        double u_draw = 2.0;
        if (!need64 && prob_step > 0.0) {
            u_draw = rng.next();
            need64 = u_draw < prob_step * ri;  // an event: redo the step's physics in FP64
        }
        prob = prob_step;
        if (need64) {
            d3 E, B;
            lcfa_fields(f, r, &E, &B, &a_eff);
            d3 n = normalize(mk3(ell.x, ell.y, ell.z));
            d3 a_perp = E - dot(E, n) * n + SPEED_OF_LIGHT * cross(n, B);
            double E_rf_sqd = norm_sqr(a_perp);
            prob = 0.0;
            if (E_rf_sqd > 0.0) {
                chi = ell.t * sqrt(E_rf_sqd) / CRITICAL_FIELD;
                prob = lcfa_pair_probability(ell, pol, chi, a_perp, dt, &pol_new);
            }
            ri = (prob * a.o.rate_increase > 0.1) ? 0.1 / prob : a.o.rate_increase;
            if (u_draw > 1.0) u_draw = rng.next();  // polarisation-resolved: first draw of the step
            if (u_draw < prob * ri) {
                double gamma_p, cos_theta, cphi;
                if (!lcfa_pair_sample(ell, pol, chi, a_perp, rng, *a.gl, &gamma_p, &cos_theta, &cphi, rej)) {
                    L.status = ST_REJECTION_CAP;
                    L.r = r;
                    return;
                }
                double sin_theta = sqrt(1.0 - cos_theta * cos_theta);
                double upm = gamma_p * sqrt(1.0 - 1.0 / (gamma_p * gamma_p));
                d3 e1 = normalize(a_perp);
                d3 e2 = cross(n, e1);
                double sp, cp;
                sincos(cphi, &sp, &cp);
                d3 p3 = upm * (cos_theta * n + (sin_theta * cp) * e1 + (sin_theta * sp) * e2);
                d3 e3 = mk3(ell.x, ell.y, ell.z) - p3;
                up = d4{sqrt(1.0 + dot(p3, p3)), p3.x, p3.y, p3.z};
                ue = d4{sqrt(1.0 + dot(e3, e3)), e3.x, e3.y, e3.z};
                frac = 1.0 / ri;
                created = true;
            }
        }
    } else {
        DbWork dbw{nullptr, 0, 32};
        if (a.dbw) {
            size_t warp = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
            dbw.base = a.dbw + warp * (size_t)a.db_cap * 5 * 32 + lane_id();
            dbw.cap = a.db_cap;
            dbw.pool = a.dbpool;
        }
        int st = lma_pair_create(f, *a.lma, dbw, r, ell, pol, dt, rng, a.o.rate_increase, &prob, &pol_new, &created,
                                 &ue, &up, &frac, &a_eff, &chi, &absorption, rej, bdf);
        if (st == LMA_DEFERRED) return;  // the step repeats once the warp has summed the rate
        if (st != ST_OK) {
            L.status = st;
            L.r = r;
            return;
        }
    }
    if (created) {
        unsigned long long slot = append_slots(a.c, 2);
        if (slot + 1 < a.s.cap) {
            unsigned long long prim = a.s.primary[L.slot];
            d4 unpol = d4{1.0, 0.0, 0.0, 0.0};
            d4 rest = d4{1.0, 0.0, 0.0, 0.0};
            spawn(a, slot, SP_ELECTRON, r, ue, rest, unpol, frac * L.weight, a_eff, chi, 0.5 * absorption, L.id, prim,
                  child_stream(L.stream, L.step, 1), L.gen + 1);
            spawn(a, slot + 1, SP_POSITRON, r, up, rest, unpol, frac * L.weight, a_eff, chi, 0.5 * absorption, L.id,
                  prim, child_stream(L.stream, L.step, 2), L.gen + 1);
            if (QUEUE) {
                publish_slot(a, slot, L.coll);
                publish_slot(a, slot + 1, L.coll);
            }
        } else {
            atomicAdd(&a.c->overflow, 2ull);
            if (QUEUE) retire_overflow(a, slot, 2);
        }
        ++*npair;
        if (frac == 1.0)
            L.decayed = true;
        else
            L.weight = L.weight * (1.0 - frac);
    }
    if (a.o.rotate_stokes && a.o.pol_resolved) L.pol = pol_new;
    L.icount += prob;
    L.r = r;
}

// Loads particle k of the wave (in its processing order) into the lane.
__device__ __forceinline__ bool lane_load_at(const WaveArgs& a, Lane& L, unsigned long long k) {
    unsigned long long i = a.lo + k;
    if (i >= a.hi) return false;
    if (a.order) i = a.lo + a.order[k];
    const Store& s = a.s;
    L.slot = i;
    L.r = get4(s.r, s.cap, i);
    L.u = get4(s.u, s.cap, i);
    L.pol = get4(s.pol, s.cap, i);
    L.weight = s.weight[i];
    L.icount = s.icount[i];
    L.work = s.work[i];
    L.stream = s.stream[i];
    L.id = s.id[i];
    L.species = s.species[i];
    L.gen = s.generation[i];
    L.status = s.status[i];
    L.flags = s.flags[i];
    L.step = 0;
    L.decayed = false;
    L.drift_cached = false;
    L.hph = SPEED_OF_LIGHT * a.o.dt / L.u.t;
    L.hh = 0.5 * SPEED_OF_LIGHT * a.o.dt / L.u.t;
    return true;
}

// The next particle of the wave for this lane alone.
__device__ __forceinline__ bool lane_load(const WaveArgs& a, Lane& L) {
    return lane_load_at(a, L, atomicAdd(&a.c->next, 1ull));
}

// The next 32 particles of the wave for the 32 lanes of a converged warp.
__device__ __forceinline__ bool warp_load(const WaveArgs& a, Lane& L) {
    unsigned long long base = 0;
    if (lane_id() == 0) base = atomicAdd(&a.c->next, 32ull);
    base = __shfl_sync(0xffffffffu, base, 0);
    return lane_load_at(a, L, base + lane_id());
}

__device__ __forceinline__ void lane_store(const WaveArgs& a, Lane& L) {
    const Store& s = a.s;
    unsigned long long i = L.slot;
    put4(s.r, s.cap, i, L.r);
    put4(s.u, s.cap, i, L.u);
    put4(s.pol, s.cap, i, L.pol);
    s.weight[i] = L.weight;
    s.icount[i] = L.icount;
    s.work[i] = L.work;
    s.status[i] = L.status;
    s.flags[i] = L.flags;
}

// This lane's DoubleBessel workspace: slot `lane` of its warp's block of
// lane-interleaved slots.
__device__ __forceinline__ DbWork lane_dbw(const WaveArgs& a) {
    DbWork w{nullptr, 0, 32};
    if (a.dbw) {
        size_t warp = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
        w.base = a.dbw + warp * (size_t)a.db_cap * 5 * 32 + lane_id();
        w.cap = a.db_cap;
        w.pool = a.dbpool;
    }
    return w;
}

// The emission deferred by lane `src` of this warp (`warp_dfr` is the
// warp's array), sampled by all 32 lanes: LP, CP with the reference's
// sampler, or CP with the learned proposal.
static __device__ __noinline__ void lp_defer_serve(const WaveArgs& a, LpDefer* warp_dfr, int src) {
    // the learned proposal's network scratch: 2 x 64 floats per warp
    __shared__ __align__(16) float s_mlp[4][2 * MLP_H];
    __syncwarp();
    LpDefer& d = warp_dfr[src];
    Draws rng = d.rng;
    int n = 0;
    double s = 0.0, theta = 0.0;
    d3 sv = mk3(0.0, 0.0, 0.0);
    uint32_t rej = 0;
    int st;
    if (!d.circular)
        st = lp_sample_warp(nlc_view(*a.lma), lane_dbw(a), d.a, d.eta, rng, &n, &s, &theta, &sv, &rej);
    else if (a.mlp.enabled)
        st = cp_sample_learned_warp(*mlp_smem(), a.mlp, nlc_view(*a.lma), s_mlp[threadIdx.x >> 5], d.a, d.eta, rng, &n,
                                    &s, &theta, &sv, &rej);
    else
        st = cp_sample_warp(nlc_view(*a.lma), d.a, d.eta, rng, &n, &s, &theta, &sv, &rej);
    __syncwarp();
    if ((int)lane_id() == src) {
        d.rng = rng;
        d.n = n, d.s = s, d.theta = theta, d.sv = sv, d.status = st, d.rej = rej;
        d.pend = 2;
    }
    __syncwarp();
}

// Emissions are sampled by the whole warp: LMA linear polarisation (with
// the DoubleBessel workspaces) and circular polarisation (the reference's
// sampler or the learned proposal); not classically.  Uniform over the
// grid: the kernel's arguments decide.
__device__ __forceinline__ bool warp_samples_emissions(const WaveArgs& a) {
    if (a.o.classical_mode) return false;
    return a.f.circular ? true : a.dbw != nullptr;
}

// The learned proposal samples on the warp from the network staged in the
// block's shared memory: staged by every thread at the kernel's start.
__device__ __forceinline__ void stage_network(const WaveArgs& a) {
    if (warp_samples_emissions(a) && a.f.circular && a.mlp.enabled) mlp_stage(a.mlp, mlp_smem());
}

// The CP Breit-Wheeler work left by lane `src` of this warp (`warp_bdf` is
// the warp's array), evaluated by all 32 lanes: the rate's harmonic sum, or
// a pair's harmonic with its s ceiling.
static __device__ __noinline__ void bw_defer_serve(const WaveArgs& a, BwDefer* warp_bdf, int src) {
    __syncwarp();
    BwDefer& d = warp_bdf[src];
    double f0, f1, ceil = 0.0;
    int n = 0;
    if (d.kind == BW_DEFER_HARMONIC) {
        bw_sample_harmonic_warp(a.lma->bw_cp_total, a.lma->bw_cp_nodes, d.a, d.eta, d.sv3, d.u, &n, &ceil, &f0, &f1);
    } else {
        bw_by_summation_warp(d.a, d.eta, &f0, &f1);
    }
    __syncwarp();
    if ((int)lane_id() == src) {
        d.f0 = f0, d.f1 = f1;
        d.n = n, d.s_ceil = ceil;
        d.pend = 2;
    }
    __syncwarp();
}

// Serves every deferred sample and sum of this warp: all 32 lanes.
__device__ __forceinline__ void warp_serve(const WaveArgs& a, LpDefer* dfr, BwDefer* bdf, bool have) {
    __syncwarp();
    if (dfr != nullptr) {
        unsigned pending = __ballot_sync(0xffffffffu, have && dfr->pend == 1);
        while (pending != 0u) {
            int src = __ffs(pending) - 1;
            pending &= pending - 1u;
            lp_defer_serve(a, dfr - lane_id(), src);
        }
    }
    if (bdf != nullptr) {
        unsigned pending = __ballot_sync(0xffffffffu, have && bdf->pend == 1);
        while (pending != 0u) {
            int src = __ffs(pending) - 1;
            pending &= pending - 1u;
            bw_defer_serve(a, bdf - lane_id(), src);
        }
    }
}

// Wave kernel.  With the LMA models in linear polarisation, emissions are
// sampled by the whole warp (LpDefer): the lanes then loop together, and
// after every round of steps the warp serves the emissions its lanes left.
template <int MODEL>
__global__ void __launch_bounds__(128) collide_wave(WaveArgs a) {
    constexpr bool LMA = MODEL == M_PLANE_WAVE || MODEL == M_FOCUSED_LASER;
    Lane L;
    uint32_t rej = 0, nemit = 0, npair = 0, maxst = 0;
    unsigned long long lsteps = 0, psteps = 0, fsteps = 0, dsteps = 0, nerr = 0;
    LpDefer* dfr = nullptr;
    BwDefer* bdf = nullptr;
    if constexpr (LMA) {
        __shared__ LpDefer s_dfr[128];
        __shared__ BwDefer s_bdf[128];
        // uniform over the grid: the kernel's arguments decide
        if (warp_samples_emissions(a)) {
            dfr = &s_dfr[threadIdx.x];
            dfr->pend = 0;
        }
        if (a.f.circular && a.o.tracking_photons) {
            bdf = &s_bdf[threadIdx.x];
            bdf->pend = 0;
        }
        stage_network(a);
    }
    bool have = a.warp_batch ? warp_load(a, L) : lane_load(a, L);
    for (;;) {
        if (have) {
            bool done;
            if (lane_stops(a, L)) {
                done = true;
            } else if (L.species != SP_PHOTON) {
                done = !(contains(a.f, L.r) && (!a.o.has_t_stop || L.r.t / SPEED_OF_LIGHT < a.o.t_stop));
                if (!done) {
                    bool fr = lepton_step<MODEL>(a, L, &rej, &nemit, dfr);
                    if (dfr == nullptr || dfr->pend != 1) {
                        ++L.step;
                        ++lsteps;
                        fsteps += fr ? 1ull : 0ull;
                        done = L.status != ST_OK;
                        if (LMA && fr && !done) {
                            uint32_t m = lma_free_run(a, L);
                            L.step += m;
                            lsteps += m;
                            fsteps += m;
                        }
                    }
                }
            } else {
                done = !(contains(a.f, L.r) && (!a.o.has_t_stop || L.r.t / SPEED_OF_LIGHT < a.o.t_stop) &&
                         !L.decayed && a.o.tracking_photons);
                if (!done && photon_drifts(a, L)) {
                    unsigned long long ds = photon_drift(a, L);
                    psteps += ds;
                    fsteps += ds;
                    dsteps += ds;
                    ds += L.step;
                    L.step = ds < 0xffffffffull ? (uint32_t)ds : 0xffffffffu;
                    done = true;
                } else if (!done) {
                    photon_step<MODEL>(a, L, &rej, &npair, bdf);
                    if (bdf == nullptr || bdf->pend != 1) {
                        ++L.step;
                        ++psteps;
                        done = L.status != ST_OK;
                    }
                }
            }
            if (done) {
                if (L.status != ST_OK) ++nerr;
                maxst = L.step > maxst ? L.step : maxst;
                // a decayed photon leaves the output, or becomes an intermediate
                if (L.species == SP_PHOTON && L.decayed) L.flags |= a.o.keep_decayed ? FLAG_INTERMEDIATE : FLAG_DROP;
                lane_store(a, L);
                have = a.warp_batch ? false : lane_load(a, L);
            }
        }
        if (a.warp_batch) {
            // the warp steps together until all 32 particles are done
            if (LMA && (dfr != nullptr || bdf != nullptr)) warp_serve(a, dfr, bdf, have);
            if (!__any_sync(0xffffffffu, have)) {
                have = warp_load(a, L);
                if (!__any_sync(0xffffffffu, have)) break;
            }
        } else if (LMA && (dfr != nullptr || bdf != nullptr)) {
            warp_serve(a, dfr, bdf, have);
            if (!__any_sync(0xffffffffu, have)) break;
        } else if (!have) {
            break;
        }
    }
    // warp reduction of the counters: one atomic per warp
    __syncwarp();
    const unsigned m = 0xffffffffu;
    for (int o = 16; o > 0; o >>= 1) {
        lsteps += __shfl_down_sync(m, lsteps, o);
        psteps += __shfl_down_sync(m, psteps, o);
        fsteps += __shfl_down_sync(m, fsteps, o);
        dsteps += __shfl_down_sync(m, dsteps, o);
        nerr += __shfl_down_sync(m, nerr, o);
        rej += __shfl_down_sync(m, rej, o);
        nemit += __shfl_down_sync(m, nemit, o);
        npair += __shfl_down_sync(m, npair, o);
    }
    maxst = __reduce_max_sync(m, maxst);
    if (lane_id() == 0) {
        if (maxst) atomicMax(&a.c->max_steps, (unsigned long long)maxst);
        atomicAdd(&a.c->lepton_steps, lsteps);
        atomicAdd(&a.c->photon_steps, psteps);
        atomicAdd(&a.c->free_steps, fsteps);
        atomicAdd(&a.c->drift_steps, dsteps);
        atomicAdd(&a.c->errors, nerr);
        atomicAdd(&a.c->rejections, (unsigned long long)rej);
        atomicAdd(&a.c->emissions, (unsigned long long)nemit);
        atomicAdd(&a.c->pair_events, (unsigned long long)npair);
    }
}

}  // namespace ptg
