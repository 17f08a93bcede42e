/* ptarmigan_gb300 — C ABI of the GB300 (sm_103a) collision-loop engine.
 *
 * This is the drop-in boundary for ptarmigan's per-particle collision loop.
 * The reference has no FFI layer; the function it replaces is the generic
 *
 *     fn collide<F: Field, R: Rng>(field: &F, incident: Particle, rng: &mut R,
 *                                  current_id: &mut u64, options: CollideOptions)
 *         -> Shower                                        (src/main.rs:134)
 *
 * mapped over a rank's primaries by src/main.rs:1118-1135 and summed into a
 * ParticleBunch.  ptg_collide_batch() takes that whole map: a batch of
 * primaries in, every surviving particle of every shower out.
 *
 * Conventions
 *   - Units follow the reference: positions are four-vectors (ct, x, y, z) in
 *     metres, momenta are normalised four-momenta u = p/(m c), Stokes vectors
 *     are [I, Q, U, V] in the reference's global basis.
 *   - Four-vectors are passed row-major, [n][4] doubles.
 *   - Errors are returned as ptg_status; the library never aborts.  A
 *     particle whose physics fails (out-of-table lookup, rejection-loop cap)
 *     is retired with a per-particle status code, mirroring the reference's
 *     panics (nonlinear_compton/mod.rs:32-35 and friends) without killing the
 *     run.
 *   - One context per host thread; calls on a context are serialised on its
 *     CUDA stream.  The context is not thread-safe.
 *   - Determinism: the same (seed, primaries, options) produce the same
 *     physics bit for bit; only the ids given to secondaries (which are
 *     drawn from a device counter) and the order of the output depend on
 *     scheduling.  Random numbers come from counter-based Philox4x32-10
 *     streams, so results are not bit-equal to the reference's Xoshiro256**.
 */
#ifndef PTARMIGAN_GB300_H
#define PTARMIGAN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PTG_ABI_VERSION 2

typedef enum {
    PTG_OK = 0,
    PTG_ERR_INVALID_ARGUMENT = 1,
    PTG_ERR_OUT_OF_TABLE = 2,    /* a rate or CDF lookup left its table */
    PTG_ERR_SANITY = 3,          /* kinematics check failed */
    PTG_ERR_REJECTION_CAP = 4,   /* a rejection loop hit its iteration cap */
    PTG_ERR_QUEUE_OVERFLOW = 5,  /* shower buffer could not grow */
    PTG_ERR_CUDA = 6,
    PTG_ERR_NO_DEVICE = 7,
    PTG_ERR_TABLES = 8,          /* table files missing or malformed */
    PTG_ERR_UNSUPPORTED = 9,     /* option combination not built yet */
    PTG_ERR_ALLOC = 10,
    PTG_ERR_TIMEOUT = 11         /* a bounded wait in the queue kernel ran out */
} ptg_status;

/* src/main.rs:1042-1060 picks the field model from (focusing, lcfa). */
typedef enum {
    PTG_PLANE_WAVE = 0,         /* LMA, 1D    field/plane_wave.rs */
    PTG_FAST_PLANE_WAVE = 1,    /* LCFA, 1D   field/fast_plane_wave.rs */
    PTG_FOCUSED_LASER = 2,      /* LMA, 3D    field/focused_laser.rs */
    PTG_FAST_FOCUSED_LASER = 3  /* LCFA, 3D   field/fast_focused_laser.rs */
} ptg_field_model;

typedef enum { PTG_POL_LINEAR = 0, PTG_POL_CIRCULAR = 1 } ptg_polarization;          /* field/mod.rs:24-28 */
typedef enum { PTG_ENV_COS2 = 0, PTG_ENV_FLATTOP = 1, PTG_ENV_GAUSSIAN = 2 } ptg_envelope; /* field/mod.rs:42-47 */
typedef enum { PTG_ELECTRON = 0, PTG_POSITRON = 1, PTG_PHOTON = 2 } ptg_species;     /* particle/mod.rs:33-38 */

/* Laser constructor arguments (main.rs:1042-1060).  n_cycles follows the
 * reference's meaning for the envelope: cos^2 and flattop take the number of
 * cycles, gaussian takes c * fwhm_duration / wavelength (main.rs:444-461). */
typedef struct {
    int32_t model;            /* ptg_field_model */
    int32_t polarization;     /* ptg_polarization */
    int32_t envelope;         /* ptg_envelope */
    int32_t finite_bandwidth; /* control:bandwidth_correction (LMA only) */
    double a0;
    double wavelength;        /* metres */
    double waist;             /* metres; ignored by plane waves */
    double n_cycles;
    double pol_angle;         /* radians; 0 for circular */
    double chirp_b;           /* plane waves only */
} ptg_laser_desc;

/* CollideOptions, src/main.rs:71-105, one field per reference field, plus
 * max_generation (tracking depth: primaries are generation 0; a particle of
 * generation > max_generation is recorded but not tracked; -1 = no limit). */
typedef struct {
    double dt_multiplier;
    double rate_increase;
    double t_stop;            /* seconds; +inf for none */
    double min_energy;        /* MeV */
    double max_angle;         /* radians */
    int32_t multiplicity;     /* -1 = no selection */
    int32_t discard_bg_e;
    int32_t discard_bg_ph;
    int32_t rr;
    int32_t tracking_photons;
    int32_t tracking_secondaries;
    int32_t keep_decayed_photons;
    int32_t pol_resolved;
    int32_t rotate_stokes_pars;
    int32_t classical;
    int32_t gaunt_factor;
    int32_t max_generation;
} ptg_collide_options;

/* A set of particles.  On input (primaries) the caller fills species, r, u,
 * pol, weight, id and parent_id; r0/u0 may be NULL (then r0 = r, u0 =
 * (1,0,0,0), as Particle::create leaves them; particle/mod.rs:108-128).  On
 * output the library fills every array. */
typedef struct {
    size_t n;
    int32_t* species;          /* [n] ptg_species */
    double* r;                 /* [n][4] position, metres */
    double* u;                 /* [n][4] normalised momentum */
    double* r0;                /* [n][4] position at creation */
    double* u0;                /* [n][4] momentum at creation */
    double* pol;               /* [n][4] Stokes vector */
    double* weight;            /* [n] */
    double* payload;           /* [n] a_eff at creation */
    double* parent_chi;        /* [n] */
    double* interaction_count; /* [n] */
    double* work;              /* [n] absorbed energy, units of m c^2 */
    uint64_t* id;              /* [n] */
    uint64_t* parent_id;       /* [n] */
    uint64_t* primary;         /* [n] output: index of the shower's primary in the input batch */
    uint64_t* stream;          /* [n] output: random-stream id (deterministic particle key) */
    int32_t* generation;       /* [n] output: 0 for primaries */
    int32_t* flags;            /* [n] output: bit 0 = decayed intermediate photon */
    int32_t* status;           /* [n] output: ptg_status of this particle */
} ptg_particles;

/* Event counters of one batch (the roofline's work model). */
typedef struct {
    uint64_t n_primaries;
    uint64_t n_out;            /* particles in the output set */
    uint64_t n_created;        /* particles ever created, primaries included */
    uint64_t lepton_steps;
    uint64_t photon_steps;
    uint64_t emissions;
    uint64_t pair_events;
    uint64_t rejections;       /* rejection-loop iterations */
    uint64_t particle_errors;  /* particles retired with status != PTG_OK */
    uint32_t waves;            /* generations launched */
    uint32_t ordered_waves;    /* of which put in order of laser phase first (three small kernels each) */
    double absorbed_energy;    /* sum of work over all particles, MeV */
    double device_ms;          /* kernel time of the batch */
    uint64_t max_steps;        /* most steps any one particle took */
    uint64_t free_steps;       /* of lepton_steps + photon_steps, those that only drifted: outside the pulse
                                  (where the field or <a^2> is below every bit the step could change), or a
                                  photon whose pair probability is zero wherever it goes */
    double wave_ms[8];         /* device time of each wave kernel (waves past the eighth add to the last
                                  entry); zero for the queue, which runs no waves */
    uint64_t drift_steps;      /* of free_steps, those of photons that only drift */
} ptg_run_stats;

typedef struct ptg_ctx ptg_ctx;

typedef struct {
    int32_t device;            /* CUDA ordinal */
    int32_t block_size;        /* 0 or 128: the collision kernels run 128 threads per block */
    int32_t blocks_per_sm;     /* 0 = occupancy maximum */
    int32_t reserved;
    size_t initial_capacity;   /* 0 = library default (particles) */
} ptg_device_cfg;

/* Library version and ABI. */
int ptg_abi_version(void);
const char* ptg_status_string(ptg_status s);
const char* ptg_last_error(void);

/* Context lifetime.  Replaces the per-rank set-up in main.rs:1036-1066. */
ptg_status ptg_context_create(const ptg_device_cfg* cfg, ptg_ctx** out);
ptg_status ptg_context_destroy(ptg_ctx* ctx);

/* Loads the rate and CDF tables (the LMA tables are data files; the LCFA
 * tables are compiled in).  dir = NULL uses the directory shipped next to
 * the library. */
ptg_status ptg_load_tables(ptg_ctx* ctx, const char* dir);

/* main.rs:1118-1135 for one batch: collide() over every primary, host
 * buffers in and out.  `out` arrays are allocated by the library (one
 * page-locked block, reused by the context's later outputs once released)
 * and must be released with ptg_particles_free().  `seed` keys the random streams
 * (the role of control:rng_seed); `id_base` is the first id handed to
 * secondaries (the reference starts current_id at the number of primaries,
 * main.rs:1070). */
ptg_status ptg_collide_batch(ptg_ctx* ctx, const ptg_laser_desc* laser, const ptg_collide_options* opts,
                             const ptg_particles* primaries, uint64_t seed, uint64_t id_base,
                             ptg_particles* out, ptg_run_stats* stats);

/* The same with every buffer already on the device: `d_primaries` holds
 * device pointers; the shower stays in library-owned device memory until
 * the next call on this context and is described by `d_out` (device
 * pointers, valid until then).  Used to time the kernels with inputs
 * resident in HBM. */
ptg_status ptg_collide_batch_device(ptg_ctx* ctx, const ptg_laser_desc* laser, const ptg_collide_options* opts,
                                    const ptg_particles* d_primaries, uint64_t seed, uint64_t id_base,
                                    ptg_particles* d_out, ptg_run_stats* stats);

/* Releases arrays allocated by ptg_collide_batch or ptg_collide_multi (the
 * block goes back to its context, or is freed if the context is gone). */
void ptg_particles_free(ptg_particles* p);

/* Allocation-free variant of ptg_collide_batch_device.  It has no
 * counterpart in the reference.
 *
 * Some callers cannot let a library call cudaMalloc: a host program whose
 * device memory is owned by another runtime's pool (a framework's caching
 * allocator, or a driver that reserves the GPU's memory at start-up) would
 * see such a call fail or fragment the pool, and cudaMalloc/cudaFree can
 * synchronise the whole device, stalling the caller's other streams.  This
 * entry point allocates nothing and needs no ptg_ctx: the caller passes the
 * primaries and the output arrays as device buffers (`d_out` rows, each at
 * least `out_capacity` long) and the CUDA stream to launch on (NULL for
 * the default stream).  It covers the LCFA field models (FastPlaneWave,
 * FastFocusedLaser); other models return PTG_ERR_UNSUPPORTED.
 *
 * Its working memory is one static device array of about 8.9 MB inside the
 * library, which every GPU that loads the library holds until the process
 * exits.  Limits: at most 4096 primaries per call (more is
 * PTG_ERR_INVALID_ARGUMENT) and at most 32768 particles in a batch's
 * showers, primaries included (more is PTG_ERR_QUEUE_OVERFLOW); a result
 * longer than out_capacity is PTG_ERR_QUEUE_OVERFLOW with the needed row
 * count in stats->n_out.  An empty batch (n = 0) gives an empty result.
 *
 * Every call looks up the array's device address in the current context
 * (cudaGetSymbolAddress, with the caller's device current) and uploads
 * 2.6 KB of constants into it on `stream`.  It waits for `stream` after
 * every wave, reading the wave's counters back to the host, so it returns
 * when its work is done.  Waves run in slot order, not in order of laser
 * phase as ptg_collide_batch_device runs its large waves; the results are
 * the same, since each particle's random stream is fixed.  All calls share
 * the array, and each call clears what must start at zero, so calls that
 * overlap on the GPU (concurrent streams or host threads) race: serialise
 * them. */
ptg_status ptg_collide_batch_noalloc(const ptg_laser_desc* laser, const ptg_collide_options* opts,
                                     const ptg_particles* d_primaries, uint64_t seed, uint64_t id_base,
                                     ptg_particles* d_out, size_t out_capacity, void* stream, ptg_run_stats* stats);

/* ------------------------------------------------ multi-collision queue ---
 * Many independent collisions in one persistent launch.  No reference
 * counterpart as one call: the reference runs one collision per process
 * (main.rs:134-289 over one beam and one laser); here each collision is
 * what a reference run with that laser, seed and beam would compute, and
 * the batch shares one shower store and one work queue on the GPU.  Each
 * collision's primaries are rows [first, first + count) of the batch's
 * primaries; its primary streams are primary_stream(id_base + i), as in
 * ptg_collide_batch with the same id_base, so a collision's shower matches
 * the single-collision call particle for particle (same seed).  The step
 * options are shared. */
typedef struct {
    ptg_laser_desc laser;
    uint64_t seed;
    uint64_t id_base;
    uint64_t first;
    uint64_t count;
} ptg_collision;

/* Launch shape of the queue kernel. */
typedef struct {
    int32_t variant;        /* 0: registers as needed; 1: capped for 3 blocks of 128 threads per SM
                               (both run whole particles lane by lane);
                               2: the single-collision kernel, for a batch of one collision
                               (larger batches run variant 0);
                               3: many collisions stepped in lockstep, one step per pass,
                               emissions sampled by the warp */
    int32_t blocks_per_sm;  /* 0 = occupancy maximum of the variant */
    int32_t chunk;          /* tickets (store slots) a lane takes per grab: 1..64 */
    int32_t use_graph;      /* replay the batch as a captured CUDA graph */
} ptg_queue_cfg;

/* Host buffers in and out: `out` is allocated by the library (free with
 * ptg_particles_free) and holds the collisions' outputs one after another;
 * collision k's rows are [out_offsets[k], out_offsets[k + 1]).  `stats`
 * ([n_coll], may be NULL) gets each collision's counts, `total` (may be
 * NULL) their sums and the batch's device time. */
ptg_status ptg_collide_multi(ptg_ctx* ctx, size_t n_coll, const ptg_collision* coll, const ptg_collide_options* opts,
                             const ptg_particles* primaries, ptg_particles* out, uint64_t* out_offsets,
                             ptg_run_stats* stats, ptg_run_stats* total);

/* Device-resident variant: primaries are device buffers; `d_out` receives
 * device pointers into the context's output buffers, valid until the
 * context's next batch; out_offsets, stats and total are host memory. */
ptg_status ptg_collide_multi_device(ptg_ctx* ctx, size_t n_coll, const ptg_collision* coll,
                                    const ptg_collide_options* opts, const ptg_particles* d_primaries,
                                    ptg_particles* d_out, uint64_t* out_offsets, ptg_run_stats* stats,
                                    ptg_run_stats* total);

/* Sets (or reads, with cfg_out) the queue kernel's launch shape. */
ptg_status ptg_queue_config(ptg_ctx* ctx, const ptg_queue_cfg* cfg, ptg_queue_cfg* cfg_out);

/* Autotuner: times the queue kernel over candidate launch shapes (variant,
 * blocks per SM, chunk) on a sample of the batch (the first
 * ceil(sample_fraction * count) primaries of each collision, device
 * buffers), keeps the fastest in the context and returns it with its
 * device time per sample batch. */
ptg_status ptg_queue_autotune(ptg_ctx* ctx, size_t n_coll, const ptg_collision* coll,
                              const ptg_collide_options* opts, const ptg_particles* d_primaries,
                              double sample_fraction, ptg_queue_cfg* best, double* best_ms);

/* Field::max_timestep (field/<model>.rs) for a laser, in seconds (or 1.0 where the
 * reference returns None), and Field::ideal_initial_z, in metres. */
ptg_status ptg_laser_timestep(const ptg_laser_desc* laser, double* dt);
ptg_status ptg_laser_initial_z(const ptg_laser_desc* laser, double* z0);

/* The CUDA stream the context launches on (a cudaStream_t). */
void* ptg_context_stream(ptg_ctx* ctx);

/* Bounds on the work any one particle, sample or wait may take.  The
 * reference has none: it steps a particle until it leaves the field and
 * repeats a rejection loop until it accepts (its samplers panic on the rare
 * inputs where they cannot), so a run there may not end; here every loop is
 * bounded and a particle that reaches a bound is retired with a
 * per-particle status, counted in ptg_run_stats.particle_errors.  Zero
 * selects the default; lower values are for exercising those exits.
 *   queue_wait_ns  any single wait of the queue kernel for a slot (default
 *                  20 s + 2 us per primary): a wait that runs out ends the
 *                  batch with PTG_ERR_TIMEOUT and leaves the context usable;
 *   step_cap       steps after which a particle still in the field is
 *                  retired with PTG_ERR_REJECTION_CAP (default 2^26; a
 *                  photon whose pair probability is zero wherever it goes
 *                  is moved to its exit in closed form and not capped);
 *   rejection_cap  iterations of any rejection loop of the collision
 *                  kernels' samplers, after which the particle is retired
 *                  with PTG_ERR_REJECTION_CAP (default 65536, at most 2^30).
 * `current` (may be NULL) receives the limits in force. */
typedef struct {
    uint64_t queue_wait_ns;
    uint32_t step_cap;
    uint32_t rejection_cap;
    uint64_t reserved;
} ptg_limits;
ptg_status ptg_context_set_limits(ptg_ctx* ctx, const ptg_limits* limits, ptg_limits* current);

/* Diagnostics entry points used by the parity tests: evaluate one field
 * model's E, B, a at n positions, and push n particles one step
 * (Field::fields / Field::push), on the device, host buffers in and out. */
ptg_status ptg_eval_fields(ptg_ctx* ctx, const ptg_laser_desc* laser, size_t n, const double* r,
                           double* E, double* B, double* a);
ptg_status ptg_push_steps(ptg_ctx* ctx, const ptg_laser_desc* laser, size_t n, double* r, double* u,
                          double rqm, double dt, int32_t eqn, int32_t nsteps, double* work);

/* Rate and sampler diagnostics (deterministic quantities checked against
 * the FP64 oracle): LCFA photon rate at (chi, gamma) and the sampled photon
 * energy for given uniforms; LCFA pair probability (unpolarised). */
ptg_status ptg_lcfa_photon_rate(ptg_ctx* ctx, size_t n, const double* chi, const double* gamma, double* rate);
ptg_status ptg_lcfa_photon_sample(ptg_ctx* ctx, size_t n, const double* chi, const double* gamma,
                                  const double* rand3, double* omega, double* theta);
ptg_status ptg_lcfa_pair_t(ptg_ctx* ctx, size_t n, const double* chi, double* t_par, double* t_perp);

/* Generalised Bessel function J(n-2..n+2, x, y) of
 * special_functions/double_bessel.rs (DoubleBessel::around, mode 0; or
 * DoubleBessel::evaluate, mode 1, which takes the saddle-point form where
 * it applies), for 0 <= x <= n sqrt 2, 0 <= y <= n / 2.  j5: [count][5]. */
ptg_status ptg_double_bessel(ptg_ctx* ctx, int32_t n, size_t count, const double* x, const double* y, int32_t mode,
                             double* j5);

/* Linearly polarised LMA emission sampler (nonlinear_compton/lp/mod.rs
 * sample, with the CDF-table harmonic index) at peak amplitude a[i] and
 * eta[i], drawing from the stream stream[i] at step `step`.
 * out7: [count][n, s, theta, 1, xi1, xi2, xi3] in the LMA basis;
 * status: [count] ptg_status per point. */
ptg_status ptg_lp_sample(ptg_ctx* ctx, size_t count, const double* a, const double* eta, uint64_t seed,
                         const uint64_t* stream, uint32_t step, double* out7, int32_t* status);

/* The same samples drawn by the warp-cooperative sampler the wave kernel
 * uses for LP emissions (each warp samples its 32 points in turn, all lanes
 * together); the results equal ptg_lp_sample's. */
ptg_status ptg_lp_sample_warp(ptg_ctx* ctx, size_t count, const double* a, const double* eta, uint64_t seed,
                              const uint64_t* stream, uint32_t step, double* out7, int32_t* status);

/* Circularly polarised LMA emission sampler (nonlinear_compton/cp/mod.rs
 * sample: the harmonic from the regenerated CDF table, v by rejection under
 * the 32-point ceiling) at rms amplitude a[i] and eta[i], drawing from
 * stream[i] at `step`; and the same drawn by the warp-cooperative sampler
 * the collision kernels use (each warp samples its 32 points in turn, all
 * lanes together), whose results equal ptg_cp_sample's.  out7 and status
 * as for ptg_lp_sample. */
ptg_status ptg_cp_sample(ptg_ctx* ctx, size_t count, const double* a, const double* eta, uint64_t seed,
                         const uint64_t* stream, uint32_t step, double* out7, int32_t* status);
ptg_status ptg_cp_sample_warp(ptg_ctx* ctx, size_t count, const double* a, const double* eta, uint64_t seed,
                              const uint64_t* stream, uint32_t step, double* out7, int32_t* status);

/* The same emissions sampled with the learned proposal in use
 * (ptg_mlp_use), as the collision kernels sample them: on each point's own
 * lane (warp = 0) or by its warp's 32 lanes together (warp = 1), with the
 * same results either way.  No reference counterpart. */
ptg_status ptg_cp_sample_learned(ptg_ctx* ctx, size_t count, const double* a, const double* eta, uint64_t seed,
                                 const uint64_t* stream, uint32_t step, int32_t warp, double* out7, int32_t* status);

/* --------------------------------------------------- learned proposal ---
 * No reference counterpart: an MLP (six features of a, eta and n; 4 layers
 * of width 64, SiLU; BF16 weights, FP32 accumulation; trained and run on the
 * tensor cores) proposes v = s / s_max for CP nonlinear Compton emission in
 * 16 bins, with an exact accept/reject against the spectrum
 * (nonlinear_compton/cp/mod.rs:17-40) and the reference's sampler as the
 * fallback wherever the learned envelope falls under the spectrum. */
typedef struct {
    uint64_t n_samples;      /* training samples drawn with the table sampler */
    int32_t batch, epochs;
    float lr, tau;           /* Adam learning rate (cosine decay); quantile of the pinball loss */
    uint64_t seed;
    double a_lo, a_hi, eta_lo, eta_hi;  /* log-uniform training domain */
} ptg_mlp_train_cfg;

typedef struct {
    float loss_first, loss_last;
    int32_t steps, reserved;
    double data_ms, train_ms;
} ptg_mlp_train_stats;

typedef struct {
    uint64_t n, seed;                   /* emissions; draws of (a, eta, n) shared by both samplers */
    double a_lo, a_hi, eta_lo, eta_hi;
    float margin, reserved;             /* ln of the envelope's safety factor */
} ptg_sampler_bench_cfg;

typedef struct {
    double plain_ms, learned_ms;            /* device times of the two samplers */
    double features_ms;                     /* the emissions' (a, eta, n) and the network's inputs: shared */
    double infer_ms;                        /* the learned path's batched inference */
    double plain_evals, learned_evals;      /* spectrum evaluations per emission */
    double acceptance;                      /* accepted / proposed under the learned envelope */
    uint64_t fallbacks;                     /* envelope under the spectrum: the reference's sampler took over */
    uint64_t exhausted;                     /* no acceptance within the learned trial cap: the envelope
                                               capped at the reference's ceiling took over */
    uint64_t errors_plain, errors_learned;  /* emissions that ended with a nonzero status */
} ptg_sampler_bench_stats;

/* Per-emission detail of the sampler benchmark (each array [n] or, for x
 * and env, [n][6] and [n][16]; any may be NULL). */
typedef struct {
    float* x;                   /* the network's inputs, [n][6] */
    float* env;                 /* its outputs */
    int32_t *status_plain, *status_learned;
    uint32_t *evals_plain, *evals_learned;
    uint32_t* fallback;         /* 0; 1 = envelope violation; 2 = trial cap; 3 = both */
} ptg_sampler_bench_detail;

/* Random initialisation; parameter access ([count] floats, get and/or
 * set); the training loop; the loss gradient of a batch ([n][8] = the six
 * inputs, bin, target) for checks; batched inference ([n][6] -> [n][16]); the
 * switch that makes the collision kernels use the network; and the sampler
 * benchmark (v_plain, v_learned: [n], may be NULL; detail may be NULL). */
ptg_status ptg_mlp_init(ptg_ctx* ctx, uint64_t seed);
ptg_status ptg_mlp_params(ptg_ctx* ctx, float* get, const float* set, int32_t* count);
ptg_status ptg_mlp_train(ptg_ctx* ctx, const ptg_mlp_train_cfg* cfg, ptg_mlp_train_stats* stats);
ptg_status ptg_mlp_grad(ptg_ctx* ctx, const float* samples, size_t n, float tau, float* grad, float* loss);
ptg_status ptg_mlp_infer(ptg_ctx* ctx, const float* x, size_t n, float* out);
ptg_status ptg_mlp_use(ptg_ctx* ctx, int32_t enabled, float margin);
/* The collision kernels propose v with the network only at harmonics n >=
 * `n` and use the reference's sampler below (both exact); *previous (may be
 * NULL) receives the setting in force before the call; n < 0 only queries.
 * The sampler benchmark always uses the network. */
ptg_status ptg_mlp_min_harmonic(ptg_ctx* ctx, int32_t n, int32_t* previous);
ptg_status ptg_sampler_bench(ptg_ctx* ctx, const ptg_sampler_bench_cfg* cfg, double* v_plain, double* v_learned,
                             const ptg_sampler_bench_detail* detail, ptg_sampler_bench_stats* stats);

/* ------------------------------------------------------ beam builder ---
 * Primary beams generated on the device: BeamBuilder::build
 * (particle/builder.rs:173-219) with GammaDistribution::sample and
 * RadialDistribution::sample (particle/dstr.rs:27-225).  Same
 * distributions; a counter-based stream per particle instead of the
 * reference's sequential RNG, so beams are statistically, not bitwise,
 * the reference's. */
typedef enum { PTG_GAMMA_NORMAL = 0, PTG_GAMMA_BREM = 1, PTG_GAMMA_CUSTOM = 2 } ptg_gamma_dstr;
typedef enum { PTG_RADIAL_NORMAL = 0, PTG_RADIAL_TRUNC_NORMAL = 1, PTG_RADIAL_UNIFORM = 2 } ptg_radial_dstr;

typedef struct {
    int32_t species;            /* ptg_species */
    int32_t gamma_dstr;         /* ptg_gamma_dstr */
    double gamma_mean;          /* Normal: mean Lorentz factor */
    double gamma_sigma;         /* Normal: rms */
    double gamma_min;           /* Brem: minimum; Custom: unused (the CDF's first node) */
    double gamma_max;           /* Brem: maximum */
    double energy_chirp;        /* Normal, Custom: gamma-z correlation (rho = -energy_chirp) */
    const double* custom_cdf;   /* Custom: host array of [len][2] (gamma, CDF) nodes, CDF from 0 to 1 */
    int32_t custom_len;         /* Custom: nodes (2..4096) */
    int32_t radial_dstr;        /* ptg_radial_dstr */
    double sigma_x, sigma_y;    /* Normal, TruncNormal: rms transverse sizes (m) */
    double x_max, y_max;        /* TruncNormal: semi-axes of the cut (m) */
    double r_max;               /* Uniform: disk radius (m) */
    double sigma_z;             /* rms length (m) */
    double rms_div;             /* rms divergence (rad) */
    double collision_angle;     /* rad */
    double collision_plane;     /* rad */
    double offset[3];           /* m */
    double initial_z;           /* Field::ideal_initial_z() + 3 sigma_z (main.rs:1064) */
    double pol[4];              /* Stokes vector of every primary */
    double weight;
} ptg_beam_desc;

/* Writes n primaries into device arrays (species, r, u, pol, weight, id,
 * parent_id of `out`, rows of 4 for four-vectors; other fields may be
 * NULL).  Particle i draws from stream (seed, first_id + i) and gets id and
 * parent id first_id + i.  Runs on the context's stream and returns after
 * the kernel has finished. */
ptg_status ptg_build_beam(ptg_ctx* ctx, const ptg_beam_desc* beam, uint64_t n, uint64_t seed, uint64_t first_id,
                          const ptg_particles* out);

/* -------------------------------------------------- distribution output ---
 * Histograms of a particle set on the device: Histogram::generate_1d and
 * generate_2d (output/hgram.rs:209-448) over the particle functions of
 * output/functions.rs, with the weights, range filter and bin and height
 * specifications of DistributionFunction (output/mod.rs:173-343). */
typedef enum {
    PTG_OUT_ANGLE_X = 0, PTG_OUT_ANGLE_Y, PTG_OUT_THETA, PTG_OUT_POLAR_ANGLE, PTG_OUT_PX, PTG_OUT_PY, PTG_OUT_PZ,
    PTG_OUT_P_PERP, PTG_OUT_R_PERP, PTG_OUT_R_X, PTG_OUT_R_Y, PTG_OUT_P_MINUS, PTG_OUT_P_PLUS, PTG_OUT_GAMMA,
    PTG_OUT_ENERGY, PTG_OUT_UNIT, PTG_OUT_X, PTG_OUT_Y, PTG_OUT_Z, PTG_OUT_RADIUS, PTG_OUT_PAYLOAD,
    PTG_OUT_PARENT_CHI, PTG_OUT_N_INTER, PTG_OUT_ABSORPTION, PTG_OUT_S1, PTG_OUT_S2, PTG_OUT_S3, PTG_OUT_POL_X,
    PTG_OUT_POL_Y, PTG_OUT_WEIGHT, PTG_OUT_HELICITY
} ptg_output_func;                                   /* output/functions.rs:10-105 */
typedef enum { PTG_WEIGHT_NUMBER = 0, PTG_WEIGHT_ENERGY, PTG_WEIGHT_POL_X, PTG_WEIGHT_POL_Y,
               PTG_WEIGHT_HELICITY } ptg_weight_func; /* output/functions.rs:244-263 */
typedef enum { PTG_BINS_AUTO = 0, PTG_BINS_LOG, PTG_BINS_FIXED_NUMBER, PTG_BINS_FIXED_SIZE } ptg_bin_spec;
typedef enum { PTG_HEIGHT_COUNT = 0, PTG_HEIGHT_DENSITY, PTG_HEIGHT_PDF } ptg_height_spec;

typedef struct {
    int32_t dim;                 /* 1 or 2 */
    int32_t species;             /* ptg_species: the particle set is the particles of this species */
    int32_t func[2];             /* ptg_output_func of each axis */
    double scale[2];             /* unit conversion of each axis: value * scale */
    int32_t weight;              /* ptg_weight_func */
    int32_t bin_spec;            /* ptg_bin_spec, both axes */
    int32_t height;              /* ptg_height_spec */
    int32_t n_bins;              /* PTG_BINS_FIXED_NUMBER */
    double bin_size;             /* PTG_BINS_FIXED_SIZE */
    int32_t filter_func;         /* ptg_output_func, or -1: no filter */
    int32_t reserved;
    double filter_min, filter_max;  /* accepted when filter_min <= func(pt) < filter_max (default units) */
} ptg_hgram_spec;

typedef struct {
    int32_t dim;
    int32_t empty;               /* 1: the set is empty (the reference writes no histogram) */
    uint64_t bins[2];
    double min[2], max[2];       /* of the (log of the, for PTG_BINS_LOG) scaled values */
    double bin_size[2];          /* 0 on an axis with a single bin */
    double bin_volume, total, unweighted_total;
    uint64_t n_counts;           /* bins[0] * bins[1] */
} ptg_hgram_info;

/* `particles` holds device arrays (rows of 4 for four-vectors); the
 * function, weight and filter read species, u, r, pol, weight, payload,
 * parent_chi, interaction_count and work as they need.  Fills `info`;
 * writes the n_counts heights (row-major as the reference's) into `counts`
 * when it is not NULL and counts_capacity >= n_counts. */
ptg_status ptg_histogram(ptg_ctx* ctx, const ptg_particles* particles, const ptg_hgram_spec* spec,
                         ptg_hgram_info* info, double* counts, uint64_t counts_capacity);

/* Sums behind the summary statistics (SummaryStatistic, output/stats.rs:
 * 265-483) over the particles of one species: with v = var_func(pt) and
 * w = weight_func(pt) (PTG_OUT_UNIT for an unweighted statistic), and
 * "within" meaning min < filter_func(pt) < max (always, without a filter),
 *   total = sum over all of v w, subtotal = sum within of v w,
 *   count = sum within of w, minimum / maximum within of v w,
 *   sum_diffs = sum within of w (v - shift), sum_sq_diffs = sum within of
 *   w (v - shift)^2, sum_cos / sum_sin = sum within of w cos v, w sin v. */
typedef struct {
    int32_t species;             /* ptg_species */
    int32_t var_func;            /* ptg_output_func */
    int32_t weight_func;         /* ptg_output_func */
    int32_t filter_func;         /* ptg_output_func, or -1 */
    double min, max;             /* filter bounds, default units, exclusive */
    double shift;
} ptg_stats_spec;

typedef struct {
    double total, subtotal, count, minimum, maximum, sum_diffs, sum_sq_diffs, sum_cos, sum_sin;
} ptg_stats_sums;

ptg_status ptg_particle_sums(ptg_ctx* ctx, const ptg_particles* particles, const ptg_stats_spec* spec,
                             ptg_stats_sums* out);

/* control:increase_pair_rate_by: auto (main.rs:294-319, 1001-1034): the
 * ratio of the photon emission and pair creation probabilities for a
 * particle of Lorentz factor `gamma` meeting the laser head on, from the
 * LCFA rates (the laser's a0 and wavelength) or, for the LMA models, the
 * LMA rates at the laser's rms amplitude (then at least 1). */
ptg_status ptg_pair_rate_increase(ptg_ctx* ctx, const ptg_laser_desc* laser, double gamma, double* ratio);

/* The LMA emission step's per-step FP32 rate beside the reference's FP64
 * rate (nonlinear_compton/cp/mod.rs:160-176, lp/mod.rs:459-553) at n points
 * (a_sqd = u.u - 1, eta): out3[3 i] the FP32 rate the step compares its
 * draw with (NaN where it does not apply and the FP64 rate decides),
 * out3[3 i + 1] the FP64 rate, out3[3 i + 2] 1 where the FP64 rate is in
 * table.  circular: the CP rate at the rms amplitude, else the LP rate at
 * the peak amplitude.  No reference counterpart (a check of the bound). */
ptg_status ptg_emission_rate_bound(ptg_ctx* ctx, size_t n, int32_t circular, const double* a_sqd, const double* eta,
                                   double* out3);

/* Measured FP64 FMA throughput of the device (TFLOP/s): the ceiling of the
 * FP64-pipe-bound collision kernels. */
ptg_status ptg_fp64_peak(ptg_ctx* ctx, double* tflops);

/* One launch of a kernel (k_fp64_fn<op>) in which every thread of one block
 * per SM calls one FP64 library function `iters` times; profiled, its FP64
 * instruction counts (less PTG_FN_NONE's) give the function's executed cost
 * per call, the weights of the collision loop's operation counts. */
typedef enum {
    PTG_FN_NONE = 0, PTG_FN_EXP = 1, PTG_FN_LOG = 2, PTG_FN_DIV = 3, PTG_FN_SQRT = 4, PTG_FN_CBRT = 5,
    PTG_FN_SINCOS = 6, PTG_FN_POW = 7, PTG_FN_ATAN2 = 8, PTG_FN_HYPOT = 9, PTG_FN_LOG1P = 10, PTG_FN_ACOS = 11
} ptg_fp64_function;
ptg_status ptg_fp64_function_kernel(ptg_ctx* ctx, int32_t op, int32_t iters);

/* Table maintenance: regenerates the CP nonlinear-Compton harmonic CDF
 * table on the device.  The reference ships it as
 * nonlinear_compton/cp/tables/cdf.rs, which is absent from its tree; this
 * is its generator (nonlinear_compton/cp/mod.rs:472-612) on the GPU.
 * cdf_out: [70*61][32][2] (eta-major grid, [n, cdf(n)] nodes);
 * total_out: [70*61] total rates, to check against the shipped totals. */
ptg_status ptg_regen_nlc_cp_cdf(ptg_ctx* ctx, double* cdf_out, double* total_out);

/* Table maintenance: regenerates the LP Breit-Wheeler mid-range harmonic
 * CDF (pair_creation/lp/tables/mid_range/cdf.rs, absent from the reference
 * tree) with its generator, pair_creation/lp/mod.rs:1063-1163
 * (TotalRate::by_summation at eta' = 2/(1 + i/4), a = 10^(-7/5 + j/20)).
 * cdf_out: [157*36][16][3] ([n, cumulative par, cumulative perp] nodes);
 * total_out: [157*36][2] totals, to check against the shipped
 * mid_range/total.rs. */
ptg_status ptg_regen_bw_lp_mid_cdf(ptg_ctx* ctx, double* cdf_out, double* total_out);

#ifdef __cplusplus
}
#endif

#endif /* PTARMIGAN_GB300_H */
