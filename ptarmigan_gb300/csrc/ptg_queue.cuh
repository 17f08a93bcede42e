// Persistent multi-collision work queue: the types shared by the engine and
// the queue kernel (ptg_queue.cu).
//
// Many independent collisions (each with its own laser, time step, seed and
// primaries) share one shower store.  One launch drains it: every lane takes
// tickets from a global cursor; ticket t is store slot t.  A slot exists once
// some lane has reserved it (n_total > t) and is readable once its producer
// has published it (ready[t] set with release semantics after the data).
// A lane whose ticket lies beyond n_total waits, bounded in time, until the
// slot is created or the queue has drained (every reserved slot finished:
// completed == n_total, read in that order).  Primaries and all generations
// of secondaries flow through the same queue, so there are no waves and no
// host round trips inside a batch.
#pragma once
#include "ptg_collide.cuh"

namespace ptg {

// Per-collision parameters, read by the lanes when they switch collision.
struct CollParams {
    FieldParams f;
    double dt;                    // max_timestep * dt_multiplier for this laser
    unsigned long long seed;
    unsigned long long id_base;   // primary streams: primary_stream(id_base + i)
};

// Per-collision event counts.
struct CollStats {
    unsigned long long lepton_steps, photon_steps, emissions, pair_events, rejections, errors;
    unsigned long long n_created, n_out;
    unsigned long long free_steps, drift_steps;
};

struct QueueArgs {
    WaveArgs base;             // store, counters, tables, shared step options
    const CollParams* coll;    // [n_coll]
    CollStats* stats;          // [n_coll]
    int n_coll;
    int chunk;                 // tickets taken per grab
    unsigned long long wait_ns;  // bound on any single wait for a slot
    // single-collision kernel: a warp takes tickets only when none of its
    // lanes holds a particle or a ticket, so that its lanes start their
    // particles together (consecutive tickets: nearby laser phases)
    int warp_batch;
};


// ------------------------------------------------------------ kernel ----
__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Warp-aggregated grab of `k` consecutive tickets per calling lane.
__device__ __forceinline__ unsigned long long grab_tickets(Counters* c, unsigned k) {
    unsigned mask = __activemask();
    unsigned leader = __ffs(mask) - 1;
    unsigned rank = __popc(mask & ((1u << lane_id()) - 1u));
    unsigned long long base = 0;
    if (lane_id() == leader) base = atomicAdd(&c->next, (unsigned long long)(k * __popc(mask)));
    base = __shfl_sync(mask, base, leader);
    return base + (unsigned long long)rank * k;
}

enum { WAIT_TIMEOUT = -1, WAIT_DRAINED = 0, WAIT_READY = 1, WAIT_SKIP = 2 };

// Waits until slot t is published (READY), lies beyond the store (SKIP:
// its producer retired it), or the queue has drained (DRAINED).  Bounded by
// `wait_ns` of wall time and by an iteration cap.
static __device__ __noinline__ int wait_slot(const WaveArgs& a, unsigned long long t, unsigned long long wait_ns) {
    unsigned long long t0 = global_ns();
    for (unsigned it = 0; it < (1u << 30); ++it) {
        unsigned long long n = ld_acquire(&a.c->n_total);
        if (t < n) {
            if (t >= a.s.cap) return WAIT_SKIP;
            for (unsigned jt = 0; jt < (1u << 30); ++jt) {
                if (ld_acquire(a.s.ready + t)) return WAIT_READY;
                if ((jt & 63u) == 63u && global_ns() - t0 > wait_ns) return WAIT_TIMEOUT;
                __nanosleep(32);
            }
            return WAIT_TIMEOUT;
        }
        unsigned long long done = ld_acquire(&a.c->completed);
        unsigned long long n2 = ld_acquire(&a.c->n_total);
        if (done == n2 && t >= n2) return WAIT_DRAINED;
        if ((it & 15u) == 15u && global_ns() - t0 > wait_ns) return WAIT_TIMEOUT;
        __nanosleep(256);
    }
    return WAIT_TIMEOUT;
}

// One look at slot t, without waiting: READY, SKIP, DRAINED or NOT_YET.
enum { POLL_NOT_YET = 3 };
__device__ __forceinline__ int poll_slot(const WaveArgs& a, unsigned long long t) {
    unsigned long long n = ld_acquire(&a.c->n_total);
    if (t < n) {
        if (t >= a.s.cap) return WAIT_SKIP;
        return ld_acquire(a.s.ready + t) ? WAIT_READY : POLL_NOT_YET;
    }
    unsigned long long done = ld_acquire(&a.c->completed);
    unsigned long long n2 = ld_acquire(&a.c->n_total);
    return (done == n2 && t >= n2) ? WAIT_DRAINED : POLL_NOT_YET;
}

struct PartCounts {
    uint32_t rej, nemit, npair;
    unsigned long long lsteps, psteps, fsteps, dsteps;
};

// main.rs:134-289 for one particle: steps it until it leaves the field,
// decays or fails.
template <int MODEL>
static __device__ __noinline__ void run_particle(const WaveArgs& a, Lane& L, PartCounts& pc) {
    for (;;) {
        bool done;
        if (lane_stops(a, L)) {
            done = true;
        } else if (L.species != SP_PHOTON) {
            done = !(contains(a.f, L.r) && (!a.o.has_t_stop || L.r.t / SPEED_OF_LIGHT < a.o.t_stop));
            if (!done) {
                bool fr = lepton_step<MODEL, true>(a, L, &pc.rej, &pc.nemit);
                pc.fsteps += fr ? 1ull : 0ull;
                ++L.step;
                ++pc.lsteps;
                done = L.status != ST_OK;
                if ((MODEL == M_PLANE_WAVE || MODEL == M_FOCUSED_LASER) && fr && !done) {
                    uint32_t m = lma_free_run(a, L);
                    L.step += m;
                    pc.lsteps += m;
                    pc.fsteps += m;
                }
            }
        } else {
            done = !(contains(a.f, L.r) && (!a.o.has_t_stop || L.r.t / SPEED_OF_LIGHT < a.o.t_stop) && !L.decayed &&
                     a.o.tracking_photons);
            if (!done && photon_drifts(a, L)) {
                unsigned long long ds = photon_drift(a, L);
                pc.psteps += ds;
                pc.fsteps += ds;
                pc.dsteps += ds;
                ds += L.step;
                L.step = ds < 0xffffffffull ? (uint32_t)ds : 0xffffffffu;
                return;
            }
            if (!done) {
                photon_step<MODEL, true>(a, L, &pc.rej, &pc.npair);
                ++L.step;
                ++pc.psteps;
                done = L.status != ST_OK;
            }
        }
        if (done) return;
    }
}

__device__ __forceinline__ void queue_load(const WaveArgs& a, Lane& L, unsigned long long i) {
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
    L.coll = s.coll[i];
    L.step = 0;
    L.decayed = false;
    L.drift_cached = false;
}

// A loaded ticket: false if it holds no particle to run (a phantom slot or
// a bad collision index), which then counts as completed.  Otherwise
// switches the lane's collision parameters if needed.
__device__ __forceinline__ bool queue_begin(const QueueArgs& q, WaveArgs& a, Lane& L, int& cur) {
    if (L.status == ST_PHANTOM || L.coll < 0 || L.coll >= q.n_coll) {
        if (L.status != ST_PHANTOM) atomicAdd(&a.c->errors, 1ull);
        __threadfence();
        atomicAdd(&a.c->completed, 1ull);
        return false;
    }
    if (L.coll != cur) {
        const CollParams& cp = q.coll[L.coll];
        a.f = cp.f;
        a.o.dt = cp.dt;
        a.seed = cp.seed;
        a.id_base = cp.id_base;
        cur = L.coll;
    }
    L.hph = SPEED_OF_LIGHT * a.o.dt / L.u.t;
    L.hh = 0.5 * SPEED_OF_LIGHT * a.o.dt / L.u.t;
    return true;
}

// A particle that has left the field, decayed or failed: its record back to
// the store, its counts to its collision, then `completed` (after its
// children, which were appended and published while it ran).
// The particle's final state written back, its failure counted, and its
// slot completed (after a fence, so that a lane that sees every slot
// completed also sees every child the particle appended).
__device__ __forceinline__ void queue_retire(const QueueArgs& q, const WaveArgs& a, Lane& L) {
    if (L.species == SP_PHOTON && L.decayed) L.flags |= a.o.keep_decayed ? FLAG_INTERMEDIATE : FLAG_DROP;
    lane_store(a, L);
    if (L.status != ST_OK) atomicAdd(&q.stats[L.coll].errors, 1ull);
    __threadfence();
    atomicAdd(&a.c->completed, 1ull);
}

// Adds a lane's event counters to collision `coll`'s statistics.
__device__ __forceinline__ void queue_count(const QueueArgs& q, int coll, const PartCounts& pc) {
    CollStats* cs = q.stats + coll;
    if (pc.lsteps) atomicAdd(&cs->lepton_steps, pc.lsteps);
    if (pc.psteps) atomicAdd(&cs->photon_steps, pc.psteps);
    if (pc.fsteps) atomicAdd(&cs->free_steps, pc.fsteps);
    if (pc.dsteps) atomicAdd(&cs->drift_steps, pc.dsteps);
    if (pc.nemit) atomicAdd(&cs->emissions, (unsigned long long)pc.nemit);
    if (pc.npair) atomicAdd(&cs->pair_events, (unsigned long long)pc.npair);
    if (pc.rej) atomicAdd(&cs->rejections, (unsigned long long)pc.rej);
}

__device__ __forceinline__ void queue_finish(const QueueArgs& q, const WaveArgs& a, Lane& L, const PartCounts& pc) {
    queue_count(q, L.coll, pc);
    queue_retire(q, a, L);
}

// One step of the lane's particle (main.rs:134-289's loop body); true when
// the particle is done.  With `bdf`, a photon step whose pair rate needs the
// harmonic sum is left to the warp and repeats after the warp has served it.
template <int MODEL>
__device__ __forceinline__ bool queue_step(const WaveArgs& a, Lane& L, PartCounts& pc, BwDefer* bdf = nullptr,
                                           LpDefer* dfr = nullptr) {
    if (lane_stops(a, L)) return true;
    if (L.species != SP_PHOTON) {
        if (!(contains(a.f, L.r) && (!a.o.has_t_stop || L.r.t / SPEED_OF_LIGHT < a.o.t_stop))) return true;
        bool fr = lepton_step<MODEL, true>(a, L, &pc.rej, &pc.nemit, dfr);
        if (dfr != nullptr && dfr->pend == 1) return false;  // the warp samples the emission first
        pc.fsteps += fr ? 1ull : 0ull;
        ++L.step;
        ++pc.lsteps;
        if (L.status != ST_OK) return true;
        if ((MODEL == M_PLANE_WAVE || MODEL == M_FOCUSED_LASER) && fr) {
            uint32_t m = lma_free_run(a, L);
            L.step += m;
            pc.lsteps += m;
            pc.fsteps += m;
        }
        return false;
    }
    if (!(contains(a.f, L.r) && (!a.o.has_t_stop || L.r.t / SPEED_OF_LIGHT < a.o.t_stop) && !L.decayed &&
          a.o.tracking_photons))
        return true;
    if (photon_drifts(a, L)) {
        unsigned long long ds = photon_drift(a, L);
        pc.psteps += ds;
        pc.fsteps += ds;
        pc.dsteps += ds;
        ds += L.step;
        L.step = ds < 0xffffffffull ? (uint32_t)ds : 0xffffffffu;
        return true;
    }
    photon_step<MODEL, true>(a, L, &pc.rej, &pc.npair, bdf);
    if (bdf != nullptr && bdf->pend == 1) return false;
    ++L.step;
    ++pc.psteps;
    return L.status != ST_OK;
}

// Steps a lane of the lockstep queue kernel takes per pass of its loop,
// between two rounds of ticket logic.
constexpr int QUEUE_STEPS_PER_PASS = 8;
// The same for the single-collision kernel.
constexpr int QUEUE_SINGLE_STEPS_PER_PASS = 16;

// Kernel variants: MINB > 1 caps the registers so that MINB blocks of 128
// threads fit on an SM (the LCFA paths need fewer registers than LMA's).
template <int MINB>
__global__ void __launch_bounds__(128, MINB) collide_queue(QueueArgs q) {
    WaveArgs a = q.base;
    int cur = -1;
    uint32_t maxst = 0;
    unsigned long long t = 0, t_end = 0;
    for (;;) {
        if (t == t_end) {
            t = grab_tickets(a.c, (unsigned)q.chunk);
            t_end = t + (unsigned long long)q.chunk;
        }
        unsigned long long ticket = t++;
        // primaries in each collision's order of laser phase (a.order)
        unsigned long long slot = (a.order && ticket < a.n_primaries) ? a.order[ticket] : ticket;
        int w = wait_slot(a, slot, q.wait_ns);
        if (w == WAIT_DRAINED) break;
        if (w == WAIT_TIMEOUT) {
            atomicAdd(&a.c->timeouts, 1ull);
            break;
        }
        if (w == WAIT_SKIP) continue;
        Lane L;
        queue_load(a, L, slot);
        if (!queue_begin(q, a, L, cur)) continue;
        PartCounts pc{0, 0, 0, 0, 0, 0, 0};
        switch (a.f.model) {
            case M_PLANE_WAVE: run_particle<M_PLANE_WAVE>(a, L, pc); break;
            case M_FAST_PLANE_WAVE: run_particle<M_FAST_PLANE_WAVE>(a, L, pc); break;
            case M_FOCUSED_LASER: run_particle<M_FOCUSED_LASER>(a, L, pc); break;
            default: run_particle<M_FAST_FOCUSED_LASER>(a, L, pc); break;
        }
        maxst = L.step > maxst ? L.step : maxst;
        queue_finish(q, a, L, pc);
    }
    if (maxst) atomicMax(&a.c->max_steps, (unsigned long long)maxst);
}

// The single-collision variant (a batch of one collision): one pass of its
// loop is up to QUEUE_SINGLE_STEPS_PER_PASS steps of every lane's particle, each
// followed by the warp's service as in collide_wave, so a lane whose
// particle ends takes its next ticket within a few steps, and the step
// code reads the collision's parameters from the kernel's parameter space
// (as collide_wave does) rather than from a per-lane copy that follows the
// lane's current collision.  A lane whose ticket is not yet published looks
// again on the next pass; the warp sleeps only when none of its lanes has a
// particle.  Every wait is bounded by q.wait_ns of wall time.  The event
// counters stay per lane over all the lane's particles and are added to
// the collision's statistics once per warp at the kernel's end.
//
// Tickets past the primaries are secondaries, mostly photons, whose steps
// are a different code path from a lepton's: a lane holding such a ticket
// starts it only once no lane of its warp is stepping a lepton, so that the
// warps that carry the last primaries (the critical path) run undivided,
// as in a wave, while warps that are free take the secondaries without a
// device-wide barrier.
template <int MODEL>
__global__ void __launch_bounds__(128) collide_queue_single(const __grid_constant__ QueueArgs q) {
    const unsigned FULL = 0xffffffffu;
    const WaveArgs& a = q.base;
    Lane L;
    PartCounts pc{0, 0, 0, 0, 0, 0, 0};
    uint32_t maxst = 0;
    bool have = false, holding = false, finished = false;
    // CP LMA photons leave their Breit-Wheeler harmonic sums to the warp
    constexpr bool LMA = MODEL == M_PLANE_WAVE || MODEL == M_FOCUSED_LASER;
    BwDefer* bdf = nullptr;
    LpDefer* dfr = nullptr;
    if constexpr (LMA) {
        __shared__ BwDefer s_bdf[128];
        __shared__ LpDefer s_dfr[128];
        if (a.f.circular && a.o.tracking_photons) {
            bdf = &s_bdf[threadIdx.x];
            bdf->pend = 0;
        }
        if (warp_samples_emissions(a)) {
            dfr = &s_dfr[threadIdx.x];
            dfr->pend = 0;
        }
        stage_network(a);
    }
    unsigned long long t = 0, t_end = 0, ticket = 0, wait_from = 0;
    for (;;) {
        if (__all_sync(FULL, finished)) break;
        bool leptons = __any_sync(FULL, have && L.species != SP_PHOTON);
        bool may_grab = !q.warp_batch || __all_sync(FULL, (!have && !holding) || finished);
        if (!have && !finished && (holding || t != t_end || may_grab)) {
            if (!holding) {
                if (t == t_end) {
                    t = grab_tickets(a.c, (unsigned)q.chunk);
                    t_end = t + (unsigned long long)q.chunk;
                }
                ticket = t++;
                holding = true;
                wait_from = global_ns();
            }
            // primaries in the batch's order of laser phase (a.order), the
            // rest in ticket order
            unsigned long long slot = (a.order && ticket < a.n_primaries) ? a.order[ticket] : ticket;
            int w = (leptons && ticket >= a.n_primaries) ? POLL_NOT_YET : poll_slot(a, slot);
            if (w == WAIT_DRAINED) {
                finished = true;
            } else if (w == WAIT_SKIP) {
                holding = false;
            } else if (w == POLL_NOT_YET) {
                if (global_ns() - wait_from > q.wait_ns) {
                    atomicAdd(&a.c->timeouts, 1ull);
                    finished = true;
                }
            } else {
                holding = false;
                queue_load(a, L, slot);
                if (L.status == ST_PHANTOM || L.coll != 0) {
                    if (L.status != ST_PHANTOM) atomicAdd(&a.c->errors, 1ull);
                    __threadfence();
                    atomicAdd(&a.c->completed, 1ull);
                } else {
                    L.hph = SPEED_OF_LIGHT * a.o.dt / L.u.t;
                    L.hh = 0.5 * SPEED_OF_LIGHT * a.o.dt / L.u.t;
                    have = true;
                }
            }
        }
        if (__all_sync(FULL, !have)) {
            __nanosleep(256);
            continue;
        }
        // up to QUEUE_SINGLE_STEPS_PER_PASS steps before the ticket logic
        // runs again (its votes then cost once per several steps); a warp
        // whose particles are all done leaves early
        for (int k = 0; k < QUEUE_SINGLE_STEPS_PER_PASS; ++k) {
            if (have && queue_step<MODEL>(a, L, pc, bdf, dfr)) {
                maxst = L.step > maxst ? L.step : maxst;
                queue_retire(q, a, L);
                have = false;
            }
            if (LMA && (bdf != nullptr || dfr != nullptr)) warp_serve(a, dfr, bdf, have);
            if (!__any_sync(FULL, have)) break;
        }
    }
    if (maxst) atomicMax(&a.c->max_steps, (unsigned long long)maxst);
    // the lane's counters over all its particles: one atomic per warp
    for (int o = 16; o > 0; o >>= 1) {
        pc.lsteps += __shfl_down_sync(FULL, pc.lsteps, o);
        pc.psteps += __shfl_down_sync(FULL, pc.psteps, o);
        pc.fsteps += __shfl_down_sync(FULL, pc.fsteps, o);
        pc.dsteps += __shfl_down_sync(FULL, pc.dsteps, o);
        pc.nemit += __shfl_down_sync(FULL, pc.nemit, o);
        pc.npair += __shfl_down_sync(FULL, pc.npair, o);
        pc.rej += __shfl_down_sync(FULL, pc.rej, o);
    }
    if (lane_id() == 0) queue_count(q, 0, pc);
}

// One step of a particle of any field model (the lockstep multi-collision
// kernel, whose lanes may hold particles of different collisions).
static __device__ __noinline__ bool queue_step_any(const WaveArgs& a, Lane& L, PartCounts& pc, BwDefer* bdf,
                                                   LpDefer* dfr) {
    switch (a.f.model) {
        case M_PLANE_WAVE: return queue_step<M_PLANE_WAVE>(a, L, pc, bdf, dfr);
        case M_FOCUSED_LASER: return queue_step<M_FOCUSED_LASER>(a, L, pc, bdf, dfr);
        case M_FAST_PLANE_WAVE: return queue_step<M_FAST_PLANE_WAVE>(a, L, pc);
        default: return queue_step<M_FAST_FOCUSED_LASER>(a, L, pc);
    }
}

// Variant 3: many collisions (the a0 scan), stepped as the single-collision
// kernel steps one: one pass of the loop is up to QUEUE_STEPS_PER_PASS
// steps of every lane's particle, a warp takes tickets together when none
// of its lanes holds a
// particle or a ticket (with q.warp_batch), and emissions, pair harmonics
// and Breit-Wheeler sums are served by the whole warp after each pass.
// Each lane keeps a copy of the step parameters that follows its current
// collision (queue_begin), as variant 0 does; a deferred emission records
// its polarisation, so that a warp may serve lanes of different
// collisions.
template <int MINB>
__global__ void __launch_bounds__(128, MINB) collide_queue_lockstep(QueueArgs q) {
    const unsigned FULL = 0xffffffffu;
    WaveArgs a = q.base;
    int cur = -1;
    Lane L;
    PartCounts pc{0, 0, 0, 0, 0, 0, 0};
    uint32_t maxst = 0;
    bool have = false, holding = false, finished = false;
    __shared__ BwDefer s_bdf[128];
    __shared__ LpDefer s_dfr[128];
    BwDefer* bdf = &s_bdf[threadIdx.x];
    bdf->pend = 0;
    // emissions go to the warp unless the rates are classical (uniform over
    // the grid: the batch's options decide)
    LpDefer* dfr = a.o.classical_mode ? nullptr : &s_dfr[threadIdx.x];
    if (dfr) dfr->pend = 0;
    if (dfr && a.mlp.enabled) mlp_stage(a.mlp, mlp_smem());
    unsigned long long t = 0, t_end = 0, ticket = 0, wait_from = 0;
    for (;;) {
        if (__all_sync(FULL, finished)) break;
        bool leptons = __any_sync(FULL, have && L.species != SP_PHOTON);
        bool may_grab = !q.warp_batch || __all_sync(FULL, (!have && !holding) || finished);
        if (!have && !finished && (holding || t != t_end || may_grab)) {
            if (!holding) {
                if (t == t_end) {
                    t = grab_tickets(a.c, (unsigned)q.chunk);
                    t_end = t + (unsigned long long)q.chunk;
                }
                ticket = t++;
                holding = true;
                wait_from = global_ns();
            }
            // primaries in each collision's order of laser phase (a.order),
            // the rest in ticket order
            unsigned long long slot = (a.order && ticket < a.n_primaries) ? a.order[ticket] : ticket;
            int w = (leptons && ticket >= a.n_primaries) ? POLL_NOT_YET : poll_slot(a, slot);
            if (w == WAIT_DRAINED) {
                finished = true;
            } else if (w == WAIT_SKIP) {
                holding = false;
            } else if (w == POLL_NOT_YET) {
                if (global_ns() - wait_from > q.wait_ns) {
                    atomicAdd(&a.c->timeouts, 1ull);
                    finished = true;
                }
            } else {
                holding = false;
                queue_load(a, L, slot);
                if (queue_begin(q, a, L, cur)) {
                    pc = PartCounts{0, 0, 0, 0, 0, 0, 0};
                    have = true;
                }
            }
        }
        if (__all_sync(FULL, !have)) {
            __nanosleep(256);
            continue;
        }
        for (int k = 0; k < QUEUE_STEPS_PER_PASS; ++k) {
            if (have && queue_step_any(a, L, pc, bdf, dfr)) {
                maxst = L.step > maxst ? L.step : maxst;
                queue_finish(q, a, L, pc);
                have = false;
            }
            warp_serve(a, dfr, bdf, have);
            if (!__any_sync(FULL, have)) break;
        }
    }
    if (maxst) atomicMax(&a.c->max_steps, (unsigned long long)maxst);
}

}  // namespace ptg
