// Host side of the engine and the extern "C" boundary declared in
// include/ptarmigan_gb300.h.
//
// A batch runs as:  primaries (row-major, host or device) -> shower store
// (SoA) -> waves of collide_wave until no particle is left to track ->
// per-shower filters of main.rs:271-282 -> compaction into row-major
// output arrays.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <dlfcn.h>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/ptarmigan_gb300.h"
#include "ptg_collide.cuh"
#include "ptg_launch.h"
#include "ptg_mlp.cuh"
#include "ptg_nlc.cuh"
#include "ptg_queue.cuh"

using namespace ptg;

static thread_local std::string g_last_error;

static ptg_status set_err(ptg_status s, const std::string& msg) {
    g_last_error = msg;
    return s;
}

#define CUDA_TRY(expr)                                                                           \
    do {                                                                                         \
        cudaError_t _e = (expr);                                                                 \
        if (_e != cudaSuccess)                                                                   \
            return set_err(PTG_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e));  \
    } while (0)

struct ptg_ctx {
    int device = 0;
    int num_sms = 0;
    int block = 128;
    int blocks_per_sm = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t ev_wa = nullptr, ev_wb = nullptr;  // around each wave launch
    // shower store
    Store s{};
    void* store_mem = nullptr;
    unsigned long long cap = 0;
    // row-major output (device) of the last batch
    void* out_mem = nullptr;
    unsigned long long out_cap = 0;
    ptg_particles d_out{};
    // staging for host primaries (row-major)
    void* in_mem = nullptr;
    unsigned long long in_cap = 0;
    ptg_particles d_in{};
    // primaries' initial momenta for the angle filter, per-shower counts
    double* init_u = nullptr;
    unsigned long long* shower_count = nullptr;
    unsigned long long init_cap = 0;
    Counters* counters = nullptr;
    Counters* h_counters = nullptr;  // pinned
    PairGL* gl = nullptr;
    LmaTables* lma_dev = nullptr;
    LmaTables lma_host{};
    // DoubleBessel workspaces for linearly polarised LMA emission
    void* dbw = nullptr;
    size_t dbw_bytes = 0;
    void* dbpool = nullptr;  // shared large J(n, x, y) slots, then their state words
    size_t dbpool_bytes = 0;
    int grid_cap = 0;  // > 0: the wave grid is capped (workspace budget)
    std::vector<void*> table_bufs;
    bool tables_loaded = false;
    // multi-collision queue: per-collision device arrays and pinned mirrors
    size_t q_cap = 0;                      // collisions the arrays hold
    CollParams* d_coll = nullptr;
    CollStats* d_cstats = nullptr;
    unsigned long long* d_qoff = nullptr;  // [q_cap + 1] loaded-index prefix of the counts
    unsigned long long* d_qfirst = nullptr;
    unsigned long long* d_qout = nullptr;  // [q_cap + 1] output offsets
    unsigned long long* d_qcursor = nullptr;
    // wave ordering by laser phase: slot permutation and bucket counters
    unsigned long long* d_order = nullptr;
    unsigned long long order_cap = 0;
    unsigned* d_buckets = nullptr;   // counts, then offsets
    unsigned* h_buckets = nullptr;   // pinned
    double* d_phase_mm = nullptr;    // per-block min/max
    double* h_phase_mm = nullptr;    // pinned
    CollParams* h_coll = nullptr;
    CollStats* h_cstats = nullptr;
    unsigned long long* h_qoff = nullptr;
    unsigned long long* h_qfirst = nullptr;
    unsigned long long* h_qout = nullptr;
    ptg_queue_cfg qcfg{0, 0, 1, 1};
    // learned CP proposal: FP32 master, Adam moments, per-block gradient
    // partials, BF16 weights (w0 w1 w2 w3 t1 t2 t3)
    float *mlp_p = nullptr, *mlp_m = nullptr, *mlp_v = nullptr, *mlp_partial = nullptr, *mlp_loss = nullptr;
    __nv_bfloat16* mlp_bf = nullptr;
    void* mlp_packed = nullptr;  // weights in fragment order for inference
    int mlp_step = 0;
    bool mlp_ready = false, mlp_enabled = false;
    int mlp_min_harmonic = MLP_MIN_HARMONIC_DEFAULT;
    // ordered waves: warps take 32 particles at a time (WaveArgs::warp_batch)
    bool warp_batch = true;
    float mlp_margin = 0.25f;
    cudaGraphExec_t q_graph = nullptr;
    std::string q_graph_key;
    ptg_limits limits{0, 0, 0, 0};
};

// ------------------------------------------------------------ helpers ---
static MlpParams mlp_params(ptg_ctx* c);

// Gauss-Laguerre node constants of the pair spectrum, and FP32 copies of the
// per-step rate tables.
static cudaError_t fill_pair_gl(PairGL* gl) {
    double nodes[32], weights[32];
    cudaError_t e = cudaMemcpyFromSymbol(nodes, PTG_GL_NODES, sizeof(nodes));
    if (e == cudaSuccess) e = cudaMemcpyFromSymbol(weights, PTG_GL_WEIGHTS, sizeof(weights));
    if (e != cudaSuccess) return e;
    for (int k = 0; k < 32; ++k) {
        double t = nodes[k];
        gl->w[k] = weights[k];
        gl->t[k] = t;
        gl->c23[k] = std::cosh(2.0 * t / 3.0);
        gl->c13_over_c1[k] = std::cosh(t / 3.0) / std::cosh(t);
        gl->c1[k] = std::cosh(t);
    }
    double ln_h[41][2], ln_t[81][3];
    e = cudaMemcpyFromSymbol(ln_h, PTG_LCFA_LN_H_CHI_TABLE, sizeof(ln_h));
    if (e == cudaSuccess) e = cudaMemcpyFromSymbol(ln_t, PTG_LCFA_LN_T_CHI_TABLE, sizeof(ln_t));
    if (e != cudaSuccess) return e;
    for (int i = 0; i < 41; ++i)
        for (int j = 0; j < 2; ++j) gl->ln_h32[i][j] = (float)ln_h[i][j];
    for (int i = 0; i < 81; ++i)
        for (int j = 0; j < 3; ++j) gl->ln_t32[i][j] = (float)ln_t[i][j];
    return cudaSuccess;
}

static FieldParams make_field(const ptg_laser_desc& d, double* dt_max) {
    FieldParams f{};
    f.model = d.model;
    f.circular = d.polarization == PTG_POL_CIRCULAR;
    f.envelope = d.envelope;
    f.finite_bandwidth = d.finite_bandwidth;
    f.a0 = d.a0;
    f.k = 2.0 * PI / d.wavelength;
    f.omega = SPEED_OF_LIGHT * f.k;
    f.duration = d.n_cycles * d.wavelength / SPEED_OF_LIGHT;
    bool focused = d.model == PTG_FOCUSED_LASER || d.model == PTG_FAST_FOCUSED_LASER;
    bool lcfa = d.model == PTG_FAST_PLANE_WAVE || d.model == PTG_FAST_FOCUSED_LASER;
    f.n_cycles = focused ? SPEED_OF_LIGHT * f.duration * f.k / (2.0 * PI) : d.n_cycles;
    f.waist = d.waist;
    f.zr = 0.5 * f.k * d.waist * d.waist;
    f.eps = d.waist / f.zr;
    f.inv_waist = 1.0 / d.waist;
    f.inv_zr = 1.0 / f.zr;
    f.inv_tau = 1.0 / (f.omega * f.duration);
    f.pol_angle = (lcfa && f.circular) ? 0.0 : d.pol_angle;
    f.cos_pa = std::cos(f.pol_angle);
    f.sin_pa = std::sin(f.pol_angle);
    f.chirp_b = focused ? 0.0 : d.chirp_b;
    f.E0 = ELECTRON_MASS * SPEED_OF_LIGHT * f.omega * d.a0 / ELEMENTARY_CHARGE;
    f.B0 = f.E0 / SPEED_OF_LIGHT;
    f.amp = (ELECTRON_MASS * SPEED_OF_LIGHT_SQD * f.k * d.a0) / ELEMENTARY_CHARGE;
    f.chi_scale = (d.model == PTG_FAST_PLANE_WAVE ? f.amp : f.E0) / CRITICAL_FIELD;
    f.eps32 = (float)f.eps;
    f.cos_pa32 = (float)f.cos_pa;
    f.sin_pa32 = (float)f.sin_pa;
    f.inv_tau32 = (float)f.inv_tau;
    f.chi_scale32 = (float)f.chi_scale;
    double nc = f.n_cycles;
    f.max_phase = d.envelope == PTG_ENV_COS2 ? PI * nc : (d.envelope == PTG_ENV_FLATTOP ? PI * (nc + 1.0) : 6.0 * PI * nc);
    f.bandwidth = 0.0;
    if (!lcfa && d.finite_bandwidth) {
        double n_fwhm = d.envelope == PTG_ENV_COS2 ? 0.36405666377387671305 * nc : nc;
        f.bandwidth = std::sqrt(0.5 * LN_2) / (PI * n_fwhm);
    }
    // Field-free region of the Gaussian FastFocusedLaser: beyond
    // |phi| = tau sqrt(ln(1e18) / (2 ln 2)) the envelope exp(-2 ln2 phi^2 /
    // tau^2) is below 1e-18, so a step's kick q E dt / (2 m c) is below
    // 1e-18 a0 omega dt and the emission probability below ~1e-19: neither
    // reaches a bit of u (|u| >= 1) nor a draw (uniforms are multiples of
    // 2^-53).  There E = B = 0 without evaluating the beam.
    f.env_cut = 0.0;
    if (d.model == PTG_FAST_FOCUSED_LASER && d.envelope == PTG_ENV_GAUSSIAN) {
        double tau = f.omega * f.duration;
        f.env_cut = tau * std::sqrt(18.0 * std::log(10.0) / (2.0 * LN_2));
    }
    // Photons that only drift.  In the LCFA models the transverse field a
    // photon sees, |E - (E.n) n + n x cB|, is at most 8 times the field
    // scale: E and cB are each below 2.2 times it (the two beams of
    // circular polarisation, the envelope's derivative and the Gaussian
    // beam's corrections of order eps^2 and beyond included).  So chi <= 8
    // ell^0 chi_scale, and a photon with ell^0 < drift_ell_max has chi <
    // 0.01 on every step, where T(chi) = 0 (lcfa/pair_creation/mod.rs:13-18):
    // its pair probability is exactly zero wherever it goes.  Chirped plane
    // waves are left out (their carrier frequency grows along the pulse).
    f.drift_ell_max = 0.0;
    if (lcfa && f.chirp_b == 0.0) f.drift_ell_max = 0.01 / (8.0 * f.chi_scale);
    // LMA models: the phase beyond which <a^2> < 2^-60 everywhere (the
    // beam factor of the focused model is at most 1).  cos^2 and flattop
    // envelopes vanish exactly beyond pi nc and pi (nc + 1); the Gaussian
    // ones fall below 2^-60 / max(1, norm a0^2).  Chirped plane waves and
    // the finite-bandwidth option (which draws a width on every step) are
    // left out.
    f.inv_w2 = 1.0 / (d.waist * d.waist);
    f.asq0 = (f.circular ? 1.0 : 0.5) * d.a0 * d.a0;
    f.env_c = 4.0 * LN_2 / ((f.omega * f.duration) * (f.omega * f.duration));
    f.lma_cut = 0.0;
    if (!lcfa && f.chirp_b == 0.0 && !d.finite_bandwidth) {
        double norm = f.circular ? 1.0 : 0.5;
        double lnk = 60.0 * LN_2 + std::log(std::fmax(1.0, norm * d.a0 * d.a0));
        if (d.envelope == PTG_ENV_COS2)
            f.lma_cut = PI * nc;
        else if (d.envelope == PTG_ENV_FLATTOP)
            f.lma_cut = PI * (nc + 1.0);
        else if (d.model == PTG_PLANE_WAVE)
            f.lma_cut = PI * nc * std::sqrt(lnk / LN_2);  // exp2(-(phase / (pi nc))^2)
        else
            f.lma_cut = f.omega * f.duration * std::sqrt(lnk / (4.0 * LN_2));  // exp(-4 ln2 phase^2 / tau^2)
    }
    // Field::max_timestep
    double dt;
    switch (d.model) {
        case PTG_PLANE_WAVE: dt = (d.envelope == PTG_ENV_FLATTOP ? 0.2 : 1.0) / (SPEED_OF_LIGHT * f.k); break;
        case PTG_FOCUSED_LASER: dt = (d.envelope == PTG_ENV_FLATTOP ? 0.2 : 1.0) / f.omega; break;
        case PTG_FAST_PLANE_WAVE: {
            double chirp = 1.0 + 2.0 * d.chirp_b * PI * d.n_cycles;
            dt = 1.0 / (SPEED_OF_LIGHT * f.k * chirp) * std::fmin(SQRT_3 / (5.0 * ALPHA_FINE * d.a0), 0.1);
            break;
        }
        default: dt = 1.0 / f.omega * std::fmin(SQRT_3 / (5.0 * ALPHA_FINE * d.a0), 0.1);
    }
    *dt_max = dt;
    return f;
}

static ptg_status check_laser(const ptg_laser_desc* d) {
    if (!d) return set_err(PTG_ERR_INVALID_ARGUMENT, "laser is NULL");
    if (d->model < 0 || d->model > 3) return set_err(PTG_ERR_INVALID_ARGUMENT, "unknown field model");
    if (d->envelope < 0 || d->envelope > 2) return set_err(PTG_ERR_INVALID_ARGUMENT, "unknown envelope");
    if (!(d->a0 > 0.0) || !(d->wavelength > 0.0) || !(d->n_cycles > 0.0))
        return set_err(PTG_ERR_INVALID_ARGUMENT, "a0, wavelength and n_cycles must be positive");
    bool focused = d->model == PTG_FOCUSED_LASER || d->model == PTG_FAST_FOCUSED_LASER;
    if (focused && !(d->waist > 0.0 && std::isfinite(d->waist)))
        return set_err(PTG_ERR_INVALID_ARGUMENT, "focused lasers need a finite waist");
    if (d->envelope == PTG_ENV_FLATTOP && d->n_cycles < 1.0)
        return set_err(PTG_ERR_INVALID_ARGUMENT, "'n_cycles' must be >= 1.0 for flattop lasers");
    return PTG_OK;
}

// ------------------------------------------------------------ kernels ---
// Primary `row` of `in` into store slot i.
__device__ __forceinline__ void load_primary(const Store& s, const ptg_particles& in, unsigned long long row,
                                             unsigned long long i, unsigned long long default_id,
                                             unsigned long long stream, double* init_u,
                                             unsigned long long* shower_count) {
    unsigned long long cap = s.cap;
    unsigned long long k = row;
    d4 r = d4{in.r[4 * k], in.r[4 * k + 1], in.r[4 * k + 2], in.r[4 * k + 3]};
    d4 u = d4{in.u[4 * k], in.u[4 * k + 1], in.u[4 * k + 2], in.u[4 * k + 3]};
    int sp = in.species[k];
    put4(s.r, cap, i, r);
    put4(s.u, cap, i, u);
    put4(s.r0, cap, i, in.r0 ? d4{in.r0[4 * k], in.r0[4 * k + 1], in.r0[4 * k + 2], in.r0[4 * k + 3]} : r);
    d4 u0 = sp == SP_PHOTON ? d4{0, 0, 0, 0} : d4{1, 0, 0, 0};
    if (in.u0) u0 = d4{in.u0[4 * k], in.u0[4 * k + 1], in.u0[4 * k + 2], in.u0[4 * k + 3]};
    put4(s.u0, cap, i, u0);
    put4(s.pol, cap, i, in.pol ? d4{in.pol[4 * k], in.pol[4 * k + 1], in.pol[4 * k + 2], in.pol[4 * k + 3]} : d4{1, 0, 0, 0});
    s.weight[i] = in.weight ? in.weight[k] : 1.0;
    s.payload[i] = 0.0;
    s.parent_chi[i] = 0.0;
    s.icount[i] = 0.0;
    s.work[i] = 0.0;
    unsigned long long id = in.id ? in.id[k] : default_id;
    s.id[i] = id;
    s.parent_id[i] = in.parent_id ? in.parent_id[k] : id;
    s.primary[i] = i;
    s.stream[i] = stream;
    s.species[i] = sp;
    s.generation[i] = 0;
    s.flags[i] = 0;
    s.status[i] = (sp < 0 || sp > 2) ? 1 : ST_OK;
    init_u[4 * i] = u.t, init_u[4 * i + 1] = u.x, init_u[4 * i + 2] = u.y, init_u[4 * i + 3] = u.z;
    shower_count[i] = 0;
}

__global__ void k_load_primaries(Store s, ptg_particles in, unsigned long long n, unsigned long long id_base,
                                 double* init_u, unsigned long long* shower_count) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    load_primary(s, in, i, i, i, primary_stream(id_base + i), init_u, shower_count);
}

struct FilterArgs {
    Store s;
    const double* init_u;
    unsigned long long* shower_count;
    unsigned long long n;
    const unsigned long long* n_live;  // if set, slots at or past *n_live are skipped as well
    double min_energy, cos_max_angle;
    int discard_bg_e, discard_bg_ph, multiplicity;
};

__device__ __forceinline__ bool filter_keep(const FilterArgs& a, unsigned long long i, bool* counted) {
    const Store& s = a.s;
    *counted = false;
    // a phantom (queue slot reserved by an append that overflowed the store)
    // holds nothing but its status
    if (s.status[i] == ST_PHANTOM) return false;
    int fl = s.flags[i];
    if (fl & FLAG_DROP) return false;
    if (fl & FLAG_INTERMEDIATE) return true;
    int gen = s.generation[i], sp = s.species[i];
    // main.rs:202-204 and :258-260: background primaries
    if (gen == 0 && sp != SP_PHOTON && a.discard_bg_e && !(s.icount[i] > 0.0)) return false;
    if (gen == 0 && sp == SP_PHOTON && a.discard_bg_ph) return false;
    if (s.status[i] != ST_OK) return true;
    // main.rs:271-276
    unsigned long long p = s.primary[i];
    d3 n0 = normalize(mk3(a.init_u[4 * p + 1], a.init_u[4 * p + 2], a.init_u[4 * p + 3]));
    d4 u = get4(s.u, s.cap, i);
    d3 n = normalize(mk3(u.x, u.y, u.z));
    bool keep = ELECTRON_MASS_MEV * u.t > a.min_energy && dot(n0, n) > a.cos_max_angle;
    *counted = keep;
    return keep;
}

__device__ __forceinline__ bool in_range(const FilterArgs& a, unsigned long long i) {
    return i < a.n && (!a.n_live || i < *a.n_live);
}

__global__ void k_filter_count(FilterArgs a) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (!in_range(a, i)) return;
    bool counted;
    filter_keep(a, i, &counted);
    if (counted) atomicAdd(&a.shower_count[a.s.primary[i]], 1ull);
}

// Store slot i into row j of a row-major output.
__device__ __forceinline__ void write_row(const ptg_particles& o, unsigned long long j, const Store& s,
                                          unsigned long long i) {
    unsigned long long cap = s.cap;
    for (int k = 0; k < 4; ++k) {
        o.r[4 * j + k] = s.r[k * cap + i];
        o.u[4 * j + k] = s.u[k * cap + i];
        o.r0[4 * j + k] = s.r0[k * cap + i];
        o.u0[4 * j + k] = s.u0[k * cap + i];
        o.pol[4 * j + k] = s.pol[k * cap + i];
    }
    o.species[j] = s.species[i];
    o.weight[j] = s.weight[i];
    o.payload[j] = s.payload[i];
    o.parent_chi[j] = s.parent_chi[i];
    o.interaction_count[j] = s.icount[i];
    o.work[j] = s.work[i];
    o.id[j] = s.id[i];
    o.parent_id[j] = s.parent_id[i];
    o.primary[j] = s.primary[i];
    o.stream[j] = s.stream[i];
    o.generation[j] = s.generation[i];
    o.flags[j] = s.flags[i];
    o.status[j] = s.status[i];
}

// filter_keep plus the multiplicity selection (main.rs:278-283), which
// drops whole showers.
__device__ __forceinline__ bool final_keep(const FilterArgs& a, unsigned long long i) {
    bool counted;
    bool keep = filter_keep(a, i, &counted);
    if (keep && a.multiplicity >= 0 && !(a.s.flags[i] & FLAG_INTERMEDIATE) &&
        a.shower_count[a.s.primary[i]] != (unsigned long long)a.multiplicity + 1)
        keep = false;
    return keep;
}

__global__ void k_compact(FilterArgs a, Counters* c, ptg_particles o, unsigned long long out_cap) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    bool keep = in_range(a, i) && final_keep(a, i);
    unsigned ballot = __ballot_sync(0xffffffffu, keep);
    if (ballot == 0) return;
    unsigned lane = threadIdx.x & 31u;
    unsigned leader = __ffs(ballot) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(&c->n_out, (unsigned long long)__popc(ballot));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (!keep) return;
    unsigned long long j = base + __popc(ballot & ((1u << lane) - 1u));
    if (j >= out_cap) return;
    write_row(o, j, a.s, i);
}

__global__ void k_sum_work(Store s, unsigned long long n, double* out) {
    double acc = 0.0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x)
        acc += s.work[i];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31u) == 0) atomicAdd(out, acc);
}

// -------------------------------------------------------- diagnostics ---
__global__ void k_eval_fields(FieldParams f, unsigned long long n, const double* r, double* E, double* B, double* a) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    d4 rr = d4{r[4 * i], r[4 * i + 1], r[4 * i + 2], r[4 * i + 3]};
    d3 e, b;
    double aa;
    if (f.model == M_FAST_PLANE_WAVE || f.model == M_FAST_FOCUSED_LASER) {
        lcfa_fields(f, rr, &e, &b, &aa);
    } else {
        e = mk3(0, 0, 0);
        b = mk3(0, 0, 0);
        aa = sqrt(lma_asq(f, rr));
    }
    E[3 * i] = e.x, E[3 * i + 1] = e.y, E[3 * i + 2] = e.z;
    B[3 * i] = b.x, B[3 * i + 1] = b.y, B[3 * i + 2] = b.z;
    a[i] = aa;
}

__global__ void k_push_steps(FieldParams f, unsigned long long n, double* r, double* u, double rqm, double dt, int eqn,
                             int nsteps, double* work) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    d4 rr = d4{r[4 * i], r[4 * i + 1], r[4 * i + 2], r[4 * i + 3]};
    d4 uu = d4{u[4 * i], u[4 * i + 1], u[4 * i + 2], u[4 * i + 3]};
    double w = 0.0;
    bool lcfa = f.model == M_FAST_PLANE_WAVE || f.model == M_FAST_FOCUSED_LASER;
    for (int s = 0; s < nsteps; ++s) {
        d4 ro, uo;
        double dw, dto;
        if (lcfa) {
            double h = 0.5 * SPEED_OF_LIGHT * dt / uu.t;
            d4 rh = d4{rr.t + h * uu.t, rr.x + h * uu.x, rr.y + h * uu.y, rr.z + h * uu.z};
            d3 E, B;
            double aa;
            lcfa_fields(f, rh, &E, &B, &aa);
            vay_push(rh, uu, E, B, rqm, dt, eqn, [](double c) { return gaunt_factor(c); }, &ro, &uo, &dw);
        } else {
            lma_push(f, rr, uu, rqm, dt, eqn, &ro, &uo, &dto, &dw);
        }
        rr = ro;
        uu = uo;
        w += dw;
    }
    r[4 * i] = rr.t, r[4 * i + 1] = rr.x, r[4 * i + 2] = rr.y, r[4 * i + 3] = rr.z;
    u[4 * i] = uu.t, u[4 * i + 1] = uu.x, u[4 * i + 2] = uu.y, u[4 * i + 3] = uu.z;
    if (work) work[i] = w;
}

__global__ void k_photon_rate(unsigned long long n, const double* chi, const double* gamma, double* rate) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i < n) rate[i] = lcfa_photon_rate(chi[i], gamma[i]);
}

__global__ void k_photon_sample(unsigned long long n, const double* chi, const double* gamma, const double* rand3,
                                double* omega, double* theta) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i < n) lcfa_photon_sample(chi[i], gamma[i], rand3[3 * i], rand3[3 * i + 1], rand3[3 * i + 2], &omega[i], &theta[i]);
}

__global__ void k_pair_t(unsigned long long n, const double* chi, double* tpar, double* tperp) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i < n) lcfa_auxiliary_t(chi[i], &tpar[i], &tperp[i]);
}

// J(n-2..n+2, x, y) per point: mode 0 by recurrence, 1 as the rate
// evaluation selects (saddle point where it applies).
__global__ void k_double_bessel(unsigned long long m, int n, int cap, const double* x, const double* y, int mode,
                                double* ws, double* j5, int* ok) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= m) return;
    DbWork w{ws + (i >> 5) * (size_t)cap * 5 * 32 + (i & 31), cap, 32};
    DbGeom g;
    double j[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    bool good = db_geom(n, cap, &g) && (mode ? db_evaluate(g, w, x[i], y[i], j) : db_around(g, w, x[i], y[i], j));
    for (int q = 0; q < 5; ++q) j5[5 * i + q] = j[q];
    ok[i] = good ? 1 : 0;
}

// One LP harmonic/s/azimuth/Stokes sample per point (the draws of the
// stream `stream[i]` at `step`).
__global__ void k_lp_sample(unsigned long long m, int cap, const LmaTables* t, const double* a, const double* eta,
                            unsigned long long seed, const unsigned long long* stream, unsigned step, double* ws,
                            double* out7, int* status) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= m) return;
    DbWork w{ws + (i >> 5) * (size_t)cap * 5 * 32 + (i & 31), cap, 32};
    Draws rng;
    rng.begin(seed, stream[i], step);
    int n = 0;
    double s = 0.0, th = 0.0;
    d3 sv = mk3(0.0, 0.0, 0.0);
    uint32_t rej = 0;
    status[i] = lp_sample(nlc_view(*t), w, a[i], eta[i], rng, &n, &s, &th, &sv, &rej);
    double* o = out7 + 7 * i;
    o[0] = n, o[1] = s, o[2] = th, o[3] = 1.0, o[4] = sv.x, o[5] = sv.y, o[6] = sv.z;
}

// The same samples with lp_sample_warp: each warp samples its 32 points
// one after another, all lanes together.
__global__ void k_lp_sample_warp(unsigned long long m, int cap, const LmaTables* t, const double* a,
                                 const double* eta, unsigned long long seed, const unsigned long long* stream,
                                 unsigned step, double* ws, double* out7, int* status) {
    unsigned long long base = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) & ~31ull;
    const unsigned lane = threadIdx.x & 31u;
    for (unsigned q = 0; q < 32u; ++q) {
        unsigned long long i = base + q;
        if (i >= m) break;  // the same for every lane of the warp
        DbWork w{ws + (base >> 5) * (size_t)cap * 5 * 32 + lane, cap, 32};
        Draws rng;
        rng.begin(seed, stream[i], step);
        int n = 0;
        double s = 0.0, th = 0.0;
        d3 sv = mk3(0.0, 0.0, 0.0);
        uint32_t rej = 0;
        int st = lp_sample_warp(nlc_view(*t), w, a[i], eta[i], rng, &n, &s, &th, &sv, &rej);
        if (lane == q) {
            status[i] = st;
            double* o = out7 + 7 * i;
            o[0] = n, o[1] = s, o[2] = th, o[3] = 1.0, o[4] = sv.x, o[5] = sv.y, o[6] = sv.z;
        }
    }
}

// ---------------------------------------------------------- storage -----
// 5 four-vectors, 5 doubles, 4 u64 and 6 32-bit fields per particle, each
// array padded to 256 B
static constexpr size_t store_bytes(unsigned long long cap) {
    return (size_t)(5 * 32 + 5 * 8 + 4 * 8 + 6 * 4) * cap + 20 * 256;
}

static void carve_store(Store* s, void* mem, unsigned long long cap) {
    char* p = (char*)mem;
    auto take = [&](size_t bytes) {
        char* q = p;
        p += (bytes + 255) & ~(size_t)255;
        return (void*)q;
    };
    s->cap = cap;
    s->r = (double*)take(32 * cap);
    s->u = (double*)take(32 * cap);
    s->r0 = (double*)take(32 * cap);
    s->u0 = (double*)take(32 * cap);
    s->pol = (double*)take(32 * cap);
    s->weight = (double*)take(8 * cap);
    s->payload = (double*)take(8 * cap);
    s->parent_chi = (double*)take(8 * cap);
    s->icount = (double*)take(8 * cap);
    s->work = (double*)take(8 * cap);
    s->id = (unsigned long long*)take(8 * cap);
    s->parent_id = (unsigned long long*)take(8 * cap);
    s->primary = (unsigned long long*)take(8 * cap);
    s->stream = (unsigned long long*)take(8 * cap);
    s->species = (int*)take(4 * cap);
    s->generation = (int*)take(4 * cap);
    s->flags = (int*)take(4 * cap);
    s->status = (int*)take(4 * cap);
    s->coll = (int*)take(4 * cap);
    s->ready = (unsigned int*)take(4 * cap);
}

static size_t particles_bytes(unsigned long long cap) {
    // 5 four-vectors, 5 doubles, 4 u64, 5 i32, each padded to 256 B
    return (size_t)(5 * 32 + 5 * 8 + 4 * 8 + 5 * 4) * cap + 19 * 256;
}

static void carve_particles(ptg_particles* p, void* mem, unsigned long long cap) {
    char* q = (char*)mem;
    auto take = [&](size_t bytes) {
        char* t = q;
        q += (bytes + 255) & ~(size_t)255;
        return (void*)t;
    };
    p->n = 0;
    p->r = (double*)take(32 * cap);
    p->u = (double*)take(32 * cap);
    p->r0 = (double*)take(32 * cap);
    p->u0 = (double*)take(32 * cap);
    p->pol = (double*)take(32 * cap);
    p->weight = (double*)take(8 * cap);
    p->payload = (double*)take(8 * cap);
    p->parent_chi = (double*)take(8 * cap);
    p->interaction_count = (double*)take(8 * cap);
    p->work = (double*)take(8 * cap);
    p->id = (uint64_t*)take(8 * cap);
    p->parent_id = (uint64_t*)take(8 * cap);
    p->primary = (uint64_t*)take(8 * cap);
    p->stream = (uint64_t*)take(8 * cap);
    p->species = (int32_t*)take(4 * cap);
    p->generation = (int32_t*)take(4 * cap);
    p->flags = (int32_t*)take(4 * cap);
    p->status = (int32_t*)take(4 * cap);
}

static ptg_status ensure_store(ptg_ctx* c, unsigned long long cap) {
    if (c->cap >= cap) return PTG_OK;
    if (c->store_mem) cudaFree(c->store_mem);
    c->store_mem = nullptr;
    c->cap = 0;
    size_t bytes = store_bytes(cap);
    if (cudaMalloc(&c->store_mem, bytes) != cudaSuccess) {
        cudaGetLastError();
        return set_err(PTG_ERR_ALLOC, "could not allocate the shower store (" + std::to_string(bytes) + " bytes)");
    }
    carve_store(&c->s, c->store_mem, cap);
    c->cap = cap;
    return PTG_OK;
}

static ptg_status ensure_out(ptg_ctx* c, unsigned long long cap) {
    if (c->out_cap >= cap) return PTG_OK;
    if (c->out_mem) cudaFree(c->out_mem);
    c->out_mem = nullptr;
    c->out_cap = 0;
    size_t bytes = particles_bytes(cap);
    if (cudaMalloc(&c->out_mem, bytes) != cudaSuccess) {
        cudaGetLastError();
        return set_err(PTG_ERR_ALLOC, "could not allocate the output buffers");
    }
    carve_particles(&c->d_out, c->out_mem, cap);
    c->out_cap = cap;
    return PTG_OK;
}

static ptg_status ensure_init(ptg_ctx* c, unsigned long long n) {
    if (c->init_cap >= n) return PTG_OK;
    if (c->init_u) cudaFree(c->init_u);
    if (c->shower_count) cudaFree(c->shower_count);
    c->init_u = nullptr;
    c->shower_count = nullptr;
    c->init_cap = 0;
    CUDA_TRY(cudaMalloc(&c->init_u, 32 * n));
    CUDA_TRY(cudaMalloc(&c->shower_count, 8 * n));
    c->init_cap = n;
    return PTG_OK;
}

// ----------------------------------------------------------- tables -----
static bool read_ptgt(const std::string& path, std::vector<double>* data, std::vector<uint32_t>* shape) {
    FILE* fp = std::fopen(path.c_str(), "rb");
    if (!fp) return false;
    char magic[4];
    uint32_t nd = 0;
    bool ok = std::fread(magic, 1, 4, fp) == 4 && std::memcmp(magic, "PTGT", 4) == 0 && std::fread(&nd, 4, 1, fp) == 1 &&
              nd > 0 && nd < 8;
    size_t n = 1;
    if (ok) {
        shape->resize(nd);
        ok = std::fread(shape->data(), 4, nd, fp) == nd;
        for (uint32_t d : *shape) n *= d;
    }
    if (ok) {
        data->resize(n);
        ok = std::fread(data->data(), 8, n, fp) == n;
    }
    std::fclose(fp);
    return ok;
}

static std::string default_table_dir() {
    Dl_info info;
    if (dladdr((void*)&default_table_dir, &info) && info.dli_fname) {
        std::string p(info.dli_fname);
        size_t slash = p.rfind('/');
        std::string dir = slash == std::string::npos ? "." : p.substr(0, slash);
        // the library lives in ptarmigan_gb300/_build/; tables in ptarmigan_gb300/tables/data
        return dir + "/../tables/data";
    }
    return "ptarmigan_gb300/tables/data";
}

// -------------------------------------------------------------- ABI -----
// Definitions below inherit C linkage from their declarations in
// include/ptarmigan_gb300.h.

int ptg_abi_version(void) { return PTG_ABI_VERSION; }

const char* ptg_status_string(ptg_status s) {
    switch (s) {
        case PTG_OK: return "ok";
        case PTG_ERR_INVALID_ARGUMENT: return "invalid argument";
        case PTG_ERR_OUT_OF_TABLE: return "lookup outside the rate/CDF table";
        case PTG_ERR_SANITY: return "kinematics sanity check failed";
        case PTG_ERR_REJECTION_CAP: return "rejection loop reached its iteration cap";
        case PTG_ERR_QUEUE_OVERFLOW: return "shower store overflow";
        case PTG_ERR_CUDA: return "CUDA error";
        case PTG_ERR_NO_DEVICE: return "no CUDA device";
        case PTG_ERR_TABLES: return "tables missing or malformed";
        case PTG_ERR_UNSUPPORTED: return "unsupported option combination";
        case PTG_ERR_ALLOC: return "device allocation failed";
        case PTG_ERR_TIMEOUT: return "a bounded device wait ran out";
    }
    return "unknown status";
}

const char* ptg_last_error(void) { return g_last_error.c_str(); }

ptg_status ptg_context_create(const ptg_device_cfg* cfg, ptg_ctx** out) {
    if (!out) return set_err(PTG_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return set_err(PTG_ERR_NO_DEVICE, "no CUDA device visible");
    }
    ptg_ctx* c = new ptg_ctx;
    c->device = cfg ? cfg->device : 0;
    if (c->device < 0 || c->device >= ndev) {
        delete c;
        return set_err(PTG_ERR_INVALID_ARGUMENT, "device ordinal out of range");
    }
    CUDA_TRY(cudaSetDevice(c->device));
    cudaDeviceProp prop;
    CUDA_TRY(cudaGetDeviceProperties(&prop, c->device));
    c->num_sms = prop.multiProcessorCount;
    if (cfg && cfg->block_size > 0 && cfg->block_size != 128) {
        delete c;
        return set_err(PTG_ERR_INVALID_ARGUMENT, "the collision kernels run 128 threads per block");
    }
    if (cfg && cfg->blocks_per_sm > 0) c->blocks_per_sm = cfg->blocks_per_sm;
    CUDA_TRY(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    CUDA_TRY(cudaEventCreate(&c->ev0));
    CUDA_TRY(cudaEventCreate(&c->ev1));
    CUDA_TRY(cudaEventCreate(&c->ev_wa));
    CUDA_TRY(cudaEventCreate(&c->ev_wb));
    CUDA_TRY(cudaMalloc(&c->counters, sizeof(Counters)));
    CUDA_TRY(cudaMallocHost(&c->h_counters, sizeof(Counters)));
    PairGL gl;
    CUDA_TRY(fill_pair_gl(&gl));
    CUDA_TRY(cudaMalloc(&c->gl, sizeof(PairGL)));
    CUDA_TRY(cudaMemcpy(c->gl, &gl, sizeof(PairGL), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMalloc(&c->lma_dev, sizeof(LmaTables)));
    CUDA_TRY(cudaMemset(c->lma_dev, 0, sizeof(LmaTables)));
    size_t init = cfg && cfg->initial_capacity ? cfg->initial_capacity : (1u << 20);
    ptg_status st = ensure_store(c, init);
    if (st != PTG_OK) {
        ptg_context_destroy(c);
        return st;
    }
    *out = c;
    return PTG_OK;
}

static void host_blocks_release(ptg_ctx* c);

ptg_status ptg_context_destroy(ptg_ctx* c) {
    if (!c) return PTG_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    host_blocks_release(c);
    cudaFree(c->store_mem);
    cudaFree(c->out_mem);
    cudaFree(c->in_mem);
    cudaFree(c->init_u);
    cudaFree(c->shower_count);
    cudaFree(c->counters);
    cudaFreeHost(c->h_counters);
    cudaFree(c->gl);
    cudaFree(c->lma_dev);
    cudaFree(c->dbw);
    cudaFree(c->dbpool);
    cudaFree(c->mlp_p), cudaFree(c->mlp_m), cudaFree(c->mlp_v), cudaFree(c->mlp_partial), cudaFree(c->mlp_loss);
    cudaFree(c->mlp_bf);
    cudaFree(c->mlp_packed);
    cudaFree(c->d_order), cudaFree(c->d_buckets), cudaFree(c->d_phase_mm);
    cudaFreeHost(c->h_buckets), cudaFreeHost(c->h_phase_mm);
    if (c->q_graph) cudaGraphExecDestroy(c->q_graph);
    cudaFree(c->d_coll);
    cudaFree(c->d_cstats);
    cudaFree(c->d_qoff);
    cudaFree(c->d_qfirst);
    cudaFree(c->d_qout);
    cudaFree(c->d_qcursor);
    cudaFreeHost(c->h_coll);
    cudaFreeHost(c->h_cstats);
    cudaFreeHost(c->h_qoff);
    cudaFreeHost(c->h_qfirst);
    cudaFreeHost(c->h_qout);
    for (void* p : c->table_bufs) cudaFree(p);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->ev_wa) cudaEventDestroy(c->ev_wa);
    if (c->ev_wb) cudaEventDestroy(c->ev_wb);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return PTG_OK;
}

void* ptg_context_stream(ptg_ctx* c) { return c ? (void*)c->stream : nullptr; }

ptg_status ptg_context_set_limits(ptg_ctx* c, const ptg_limits* limits, ptg_limits* current) {
    if (!c) return set_err(PTG_ERR_INVALID_ARGUMENT, "ctx is NULL");
    if (limits) {
        if (limits->rejection_cap > (1u << 30)) return set_err(PTG_ERR_INVALID_ARGUMENT, "rejection cap above 2^30");
        c->limits = *limits;
    }
    if (current) *current = c->limits;
    return PTG_OK;
}

// The CP harmonic CDF's nodes in the coordinates of its inversion
// (nonlinear_compton/cp/tables/mod.rs:47-121), once per load.
__global__ void k_cp_cdf_log(const double* cdf, double* out, unsigned long long nodes) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= nodes) return;
    out[2 * i] = log(cdf[2 * i]);
    out[2 * i + 1] = cp_cdf_log_node(cdf[2 * i + 1]);
}

// K(eta) of the emission rate a^2 K(eta) below the rate tables' smallest
// amplitude: circular polarisation, nonlinear_compton/cp/mod.rs:160-176
// (a the rms amplitude); linear, the linear rate of lp/mod.rs:459-553 for
// eta > 1e-3 (a the peak amplitude).  Upper bounds per cell of ln eta: the
// largest of 65 values across the cell (K increases with eta), raised by
// 2^-8 and rounded up to FP32.
static double small_a_factor(bool circular, double eta) {
    double q = 1.0 + 2.0 * eta;
    if (circular)
        return (2.0 + 8.0 * eta + 9.0 * eta * eta + eta * eta * eta) / (2.0 * eta * q * q) -
               (2.0 + 2.0 * eta - eta * eta) * std::log(q) / (4.0 * eta * eta);
    return (0.5 + 4.0 / eta - 0.5 / (q * q) + (1.0 - 2.0 / eta - 2.0 / (eta * eta)) * std::log(q)) / 8.0;
}

static std::vector<float> small_a_bounds(bool circular) {
    std::vector<float> out(SMALL_A_CELLS);
    const double w = (SMALL_A_LN_ETA1 - SMALL_A_LN_ETA0) / SMALL_A_CELLS;
    for (int j = 0; j < SMALL_A_CELLS; ++j) {
        double mx = 0.0;
        for (int k = 0; k <= 64; ++k) {
            double le = SMALL_A_LN_ETA0 + (j + k / 64.0) * w;
            mx = std::max(mx, small_a_factor(circular, std::exp(le)));
        }
        double b = mx * (1.0 + 1.0 / 256.0);
        float f = (float)b;
        if ((double)f < b) f = std::nextafter(f, INFINITY);
        out[j] = f;
    }
    return out;
}

ptg_status ptg_load_tables(ptg_ctx* c, const char* dir) {
    if (!c) return set_err(PTG_ERR_INVALID_ARGUMENT, "ctx is NULL");
    std::string d = dir ? dir : default_table_dir();
    struct Want {
        const char* name;
        const double** slot;
        size_t count;
        bool required;
    } wants[] = {
        {"nlc_lp_rate", &c->lma_host.nlc_lp_rate, 68 * 61, true},
        {"nlc_lp_cdf", &c->lma_host.nlc_lp_cdf, 4148 * 16 * 2, true},
        {"nlc_cp_rate", &c->lma_host.nlc_cp_rate, 70 * 61, true},
        {"nlc_cp_cdf", &c->lma_host.nlc_cp_cdf, 4270 * 32 * 2, false},
        {"nlc_lp_classical_rate", &c->lma_host.nlc_lp_cl_rate, 61, true},
        {"nlc_cp_classical_rate", &c->lma_host.nlc_cp_cl_rate, 61, true},
        {"bw_cp_total", &c->lma_host.bw_cp_total, 121 * 74 * 2, true},
        {"bw_lp_total", &c->lma_host.bw_lp_total, 61 * 25 * 2, true},
        {"bw_lp_cdf", &c->lma_host.bw_lp_cdf, 1525 * 16 * 3, true},
        {"bw_lp_mid_total", &c->lma_host.bw_lp_mid_total, 157 * 36 * 2, true},
        {"bw_lp_mid_cdf", &c->lma_host.bw_lp_mid_cdf, 5652 * 16 * 3, false},
        {"nlc_cp_classical_cdf", &c->lma_host.nlc_cp_cl_cdf, 61 * 32 * 2, true},
        {"nlc_lp_classical_cdf", &c->lma_host.nlc_lp_cl_cdf, 61 * 16 * 2, true},
    };
    CUDA_TRY(cudaSetDevice(c->device));
    // all or nothing: the context keeps its tables unless every file reads
    LmaTables host = c->lma_host;
    std::vector<void*> bufs;
    auto fail = [&](ptg_status st, const std::string& msg) {
        for (void* p : bufs) cudaFree(p);
        return set_err(st, msg);
    };
    for (auto& w : wants) {
        std::vector<double> data;
        std::vector<uint32_t> shape;
        std::string path = d + "/" + w.name + ".ptgt";
        const double** slot = (const double**)((char*)&host + ((char*)w.slot - (char*)&c->lma_host));
        if (!read_ptgt(path, &data, &shape)) {
            if (w.required) return fail(PTG_ERR_TABLES, "cannot read table " + path);
            *slot = nullptr;
            continue;
        }
        if (data.size() != w.count) return fail(PTG_ERR_TABLES, "table " + path + " has the wrong size");
        for (double v : data)
            if (std::isnan(v)) return fail(PTG_ERR_TABLES, "table " + path + " holds a NaN");
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, 8 * data.size());
        if (e != cudaSuccess) return fail(PTG_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        bufs.push_back(p);
        e = cudaMemcpy(p, data.data(), 8 * data.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return fail(PTG_ERR_CUDA, std::string("cudaMemcpy: ") + cudaGetErrorString(e));
        *slot = (const double*)p;
        // FP32 copies of the emission rate tables (the per-step bound)
        const float** slot32 = nullptr;
        if (std::strcmp(w.name, "nlc_cp_rate") == 0) slot32 = &host.nlc_cp_rate32;
        if (std::strcmp(w.name, "nlc_lp_rate") == 0) slot32 = &host.nlc_lp_rate32;
        if (slot32) {
            std::vector<float> f32(data.begin(), data.end());
            void* q = nullptr;
            e = cudaMalloc(&q, 4 * f32.size());
            if (e != cudaSuccess) return fail(PTG_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
            bufs.push_back(q);
            e = cudaMemcpy(q, f32.data(), 4 * f32.size(), cudaMemcpyHostToDevice);
            if (e != cudaSuccess) return fail(PTG_ERR_CUDA, std::string("cudaMemcpy: ") + cudaGetErrorString(e));
            *slot32 = (const float*)q;
        }
    }
    // node positions of the CP Breit-Wheeler table, with the host's
    // exponential (the reference evaluates them with its libm on the host)
    {
        std::vector<double> nodes(74 + 121);
        for (int i = 0; i < 74; ++i) nodes[i] = std::exp(PTG_BW_CP_LN_MIN_A + i * PTG_BW_CP_LN_A_STEP);
        for (int j = 0; j < 121; ++j) nodes[74 + j] = std::exp(PTG_BW_CP_LN_MIN_ETA + j * PTG_BW_CP_LN_ETA_STEP);
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, 8 * nodes.size());
        if (e != cudaSuccess) return fail(PTG_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        bufs.push_back(q);
        e = cudaMemcpy(q, nodes.data(), 8 * nodes.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return fail(PTG_ERR_CUDA, std::string("cudaMemcpy: ") + cudaGetErrorString(e));
        host.bw_cp_nodes = (const double*)q;
    }
    // upper bounds of the small-amplitude rate factors K(eta) per cell of
    // ln eta (the per-step FP32 bound below the rate tables)
    for (int pol = 0; pol < 2; ++pol) {
        std::vector<float> k32 = small_a_bounds(pol == 0);
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, 4 * k32.size());
        if (e != cudaSuccess) return fail(PTG_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        bufs.push_back(q);
        e = cudaMemcpy(q, k32.data(), 4 * k32.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return fail(PTG_ERR_CUDA, std::string("cudaMemcpy: ") + cudaGetErrorString(e));
        (pol == 0 ? host.nlc_cp_small32 : host.nlc_lp_small32) = (const float*)q;
    }
    host.nlc_cp_cdf_log = nullptr;
    if (host.nlc_cp_cdf) {
        const unsigned long long nodes = 4270ull * 32;
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, 16 * nodes);
        if (e != cudaSuccess) return fail(PTG_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        bufs.push_back(q);
        k_cp_cdf_log<<<(unsigned)((nodes + 255) / 256), 256>>>(host.nlc_cp_cdf, (double*)q, nodes);
        e = cudaDeviceSynchronize();
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e != cudaSuccess) return fail(PTG_ERR_CUDA, std::string("CDF transform: ") + cudaGetErrorString(e));
        host.nlc_cp_cdf_log = (const double*)q;
    }
    CUDA_TRY(cudaMemcpy(c->lma_dev, &host, sizeof(LmaTables), cudaMemcpyHostToDevice));
    c->lma_host = host;
    for (void* p : bufs) c->table_bufs.push_back(p);
    c->tables_loaded = true;
    return PTG_OK;
}

ptg_status ptg_laser_timestep(const ptg_laser_desc* laser, double* dt) {
    ptg_status st = check_laser(laser);
    if (st != PTG_OK) return st;
    make_field(*laser, dt);
    return PTG_OK;
}

ptg_status ptg_laser_initial_z(const ptg_laser_desc* d, double* z0) {
    ptg_status st = check_laser(d);
    if (st != PTG_OK) return st;
    double dt;
    FieldParams f = make_field(*d, &dt);
    double wl = 2.0 * PI / f.k;
    double nc = f.n_cycles;
    *z0 = d->envelope == PTG_ENV_COS2 ? 0.5 * wl * nc : (d->envelope == PTG_ENV_FLATTOP ? 0.5 * wl * (nc + 1.0) : 2.0 * wl * nc);
    return PTG_OK;
}

static int grid_for(ptg_ctx* c, const void* kernel) {
    int per_sm = c->blocks_per_sm;
    if (per_sm <= 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, c->block, 0);
        if (per_sm <= 0) per_sm = 1;
    }
    return per_sm * c->num_sms;
}

static const void* wave_kernel(int model) {
    return (model == M_PLANE_WAVE || model == M_FOCUSED_LASER) ? wave_kernel_lma(model) : wave_kernel_lcfa(model);
}

static cudaError_t launch_wave_model(ptg_ctx* c, const WaveArgs& a) {
    int grid = grid_for(c, wave_kernel(a.f.model));
    if (c->grid_cap > 0 && grid > c->grid_cap) grid = c->grid_cap;
    unsigned long long n = a.hi - a.lo;
    int threads = 128;
    if (n < (unsigned long long)grid * 128ull) {
        // a wave smaller than the resident grid: one-warp blocks, so that
        // its warps spread over every SM instead of filling the first few
        // (the same lanes: the workspaces cover grid x 4 warps)
        threads = 32;
        grid = (int)std::min<unsigned long long>((n + 31) / 32, (unsigned long long)grid * 4ull);
    }
    if (grid < 1) grid = 1;
    if (a.f.model == M_PLANE_WAVE || a.f.model == M_FOCUSED_LASER)
        return launch_wave_lma(a.f.model, grid, threads, c->stream, a);
    return launch_wave_lcfa(a.f.model, grid, threads, c->stream, a);
}

// Linearly polarised LMA emission evaluates J(n, x, y) by recurrence in a
// per-lane workspace of 40 bytes per order.  Slots are sized for harmonics up
// to 1.5x the reference's harmonic sum limit at 1.05 a0 (its eta -> 0 bound);
// a sampled order beyond that retires the particle with PTG_ERR_UNSUPPORTED.
// The workspace stays within min(8 GiB, free / 4), which may cap the grid.
static ptg_status ensure_dbw(ptg_ctx* c, double a0, int grid_wanted, WaveArgs* a, int* grid_out) {
    double A = 1.05 * a0;
    int n_cap = (int)std::ceil(1.5 * (6.0 * (1.0 + A * A) + 2.0 * A * A * A)) + 16;
    int cap = db_len_for(n_cap);
    size_t per_block = (size_t)cap * 5 * 32 * sizeof(double) * (size_t)((c->block + 31) / 32);
    size_t free_b = 0, total_b = 0;
    CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    size_t budget = std::min<size_t>((size_t)8 << 30, (free_b + c->dbw_bytes + c->dbpool_bytes) / 4);
    // the shared pool: harmonics of pair creation down to the smallest eta
    // where the LP rate is not negligible (pair_creation/lp/mod.rs:371-374),
    // clipped to the tables' eta >= 0.002
    double l = std::log10(A) + 2.0;
    double eta_min = std::max(std::pow(10.0, -1.0 - l * l / 4.5), 0.002);
    int p_min, p_max;
    lpp_sum_limits(A, eta_min, &p_min, &p_max);
    int pool_cap = db_len_for(std::max(p_max + 16, n_cap));
    size_t slot_bytes = (size_t)pool_cap * 5 * sizeof(double);
    int slots = (int)std::min<size_t>(64, (budget / 4) / slot_bytes);
    size_t pool_bytes = slots > 0 ? slot_bytes * (size_t)slots + 256 + 4 * (size_t)slots : 0;
    size_t max_blocks = (budget - std::min(budget, pool_bytes)) / per_block;
    if (max_blocks < 1)
        return set_err(PTG_ERR_ALLOC, "no room for one block of LP LMA workspaces at a0 = " + std::to_string(a0));
    int grid = grid_wanted;
    if ((size_t)grid > max_blocks) grid = (int)max_blocks;
    size_t need = per_block * (size_t)grid;
    if (need > c->dbw_bytes) {
        cudaFree(c->dbw);
        c->dbw = nullptr;
        c->dbw_bytes = 0;
        if (cudaMalloc(&c->dbw, need) != cudaSuccess) {
            cudaGetLastError();
            return set_err(PTG_ERR_ALLOC, "cannot allocate LP LMA workspaces (" + std::to_string(need) + " bytes)");
        }
        c->dbw_bytes = need;
    }
    if (pool_bytes > c->dbpool_bytes) {
        cudaFree(c->dbpool);
        c->dbpool = nullptr;
        c->dbpool_bytes = 0;
        if (cudaMalloc(&c->dbpool, pool_bytes) != cudaSuccess) {
            cudaGetLastError();
            return set_err(PTG_ERR_ALLOC, "cannot allocate the shared J(n, x, y) pool");
        }
        c->dbpool_bytes = pool_bytes;
    }
    a->dbw = (double*)c->dbw;
    a->db_cap = cap;
    a->dbpool = DbPool{};
    if (slots > 0) {
        size_t state_off = (slot_bytes * (size_t)slots + 255) & ~(size_t)255;
        a->dbpool.base = (double*)c->dbpool;
        a->dbpool.state = (unsigned*)((char*)c->dbpool + state_off);
        a->dbpool.cap = pool_cap;
        a->dbpool.slots = slots;
        CUDA_TRY(cudaMemsetAsync(a->dbpool.state, 0, 4 * (size_t)slots, c->stream));
    }
    *grid_out = grid;
    return PTG_OK;
}

// The option checks of main.rs:339-400 for one laser; loads the LMA tables
// when the model needs them.
static ptg_status check_run(ptg_ctx* c, const ptg_laser_desc* laser, const ptg_collide_options* o) {
    ptg_status st = check_laser(laser);
    if (st != PTG_OK) return st;
    if (!o) return set_err(PTG_ERR_INVALID_ARGUMENT, "options is NULL");
    bool lcfa = laser->model == PTG_FAST_PLANE_WAVE || laser->model == PTG_FAST_FOCUSED_LASER;
    if (o->gaunt_factor && !lcfa)
        return set_err(PTG_ERR_INVALID_ARGUMENT, "Gaunt factor correction is only available under the LCFA");
    if (!(o->rate_increase >= 1.0)) return set_err(PTG_ERR_INVALID_ARGUMENT, "increase in pair creation rate must be >= 1.0");
    if (o->rate_increase > 1.0 && o->multiplicity >= 0)
        return set_err(PTG_ERR_INVALID_ARGUMENT, "event biasing is incompatible with multiplicity selection");
    if (!lcfa && !c->tables_loaded) {
        st = ptg_load_tables(c, nullptr);
        if (st != PTG_OK) return st;
    }
    return PTG_OK;
}

// StepOptions from the collision options (dt is set per laser).
static void fill_step_options(const ptg_collide_options& o, StepOptions* so) {
    so->t_stop = o.t_stop;
    so->has_t_stop = std::isfinite(o.t_stop) ? 1 : 0;
    so->rate_increase = o.rate_increase;
    so->eqn = (o.classical && o.rr) ? (o.gaunt_factor ? EQN_MODIFIED_LL : EQN_LL) : EQN_LORENTZ;
    so->classical_mode = o.classical && !o.gaunt_factor;
    so->classical = o.classical;
    so->electron_recoils = !o.classical && o.rr;
    so->tracking_photons = o.tracking_photons;
    so->pol_resolved = o.pol_resolved;
    so->rotate_stokes = o.rotate_stokes_pars;
    so->tracking_secondaries = o.tracking_secondaries;
    so->max_generation = o.max_generation;
    so->keep_decayed = o.keep_decayed_photons;
    so->step_cap = STEP_CAP;
    so->rej_cap = REJECTION_CAP;
}

// The context's limits (ptg_context_set_limits) over the defaults.
static void apply_limits(const ptg_ctx* c, StepOptions* so) {
    if (c->limits.step_cap) so->step_cap = c->limits.step_cap;
    if (c->limits.rejection_cap) so->rej_cap = (int)c->limits.rejection_cap;
}

// ----------------------------------------------------- wave ordering ---
// A wave's lanes take particles in order of their laser phase k (t - z)
// (furthest from the pulse first): the lanes of a warp then enter and leave
// the pulse together, so the field evaluations and emission steps run with
// full warps, and the longest trajectories start first.  A counting sort
// over WAVE_BUCKETS phase buckets.
constexpr int WAVE_BUCKETS = 4096;
constexpr int WAVE_ORDER_BLOCKS = 256;
constexpr unsigned long long WAVE_ORDER_MIN = 2048;  // smaller waves run in slot order

// t - z of particle k of the range: store slots lo + k (component-major),
// or, with rows != NULL, row-major input rows lo + k.
struct WaveKeys {
    Store s;
    const double* rows;
    __device__ __forceinline__ double key(unsigned long long i) const {
        return rows ? rows[4 * i] - rows[4 * i + 3] : s.r[0 * s.cap + i] - s.r[3 * s.cap + i];
    }
};

__global__ void k_wave_key_range(WaveKeys s, unsigned long long lo, unsigned long long n, double* mm) {
    __shared__ double smin[256], smax[256];
    double mn = HUGE_VAL, mx = -HUGE_VAL;
    for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < n;
         k += (unsigned long long)gridDim.x * blockDim.x) {
        double v = s.key(lo + k);
        mn = fmin(mn, v), mx = fmax(mx, v);
    }
    smin[threadIdx.x] = mn, smax[threadIdx.x] = mx;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            smin[threadIdx.x] = fmin(smin[threadIdx.x], smin[threadIdx.x + w]);
            smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + w]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) mm[2 * blockIdx.x] = smin[0], mm[2 * blockIdx.x + 1] = smax[0];
}

__device__ __forceinline__ int wave_bucket(double v, double mn, double inv_width) {
    double b = (v - mn) * inv_width;  // NaN keys go to bucket 0
    return b > 0.0 ? (b < (double)(WAVE_BUCKETS - 1) ? (int)b : WAVE_BUCKETS - 1) : 0;
}

__global__ void k_wave_bucket_count(WaveKeys s, unsigned long long lo, unsigned long long n, double mn,
                                    double inv_width, unsigned* counts) {
    unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (k < n) atomicAdd(&counts[wave_bucket(s.key(lo + k), mn, inv_width)], 1u);
}

__global__ void k_wave_bucket_scatter(WaveKeys s, unsigned long long lo, unsigned long long n, double mn,
                                      double inv_width, unsigned* offsets, unsigned long long* order,
                                      unsigned long long base) {
    unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (k >= n) return;
    unsigned pos = atomicAdd(&offsets[wave_bucket(s.key(lo + k), mn, inv_width)], 1u);
    order[pos] = base + k;
}

__global__ void k_iota(unsigned long long* out, unsigned long long n) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i < n) out[i] = i;
}

static bool order_range(ptg_ctx* c, const WaveKeys& s, unsigned long long lo, unsigned long long hi,
                        unsigned long long* out, unsigned long long base);

static bool ensure_order(ptg_ctx* c, unsigned long long n) {
    if (c->order_cap >= n) return true;
    cudaFree(c->d_order);
    c->d_order = nullptr;
    c->order_cap = 0;
    if (cudaMalloc(&c->d_order, 8 * n) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    c->order_cap = n;
    return true;
}

// Fills c->d_order for slots [lo, hi) with offsets from lo (synchronises
// the stream).  Returns false if the wave keeps slot order.
static bool order_wave(ptg_ctx* c, const WaveKeys& s, unsigned long long lo, unsigned long long hi) {
    unsigned long long n = hi - lo;
    if (n < WAVE_ORDER_MIN || n > 0xffffffffull) return false;
    if (!ensure_order(c, n)) return false;
    return order_range(c, s, lo, hi, c->d_order, 0);
}

// A batch of collisions whose primaries fill slots [off_k, off_k + count_k)
// from input rows [first_k, ...): c->d_order maps ticket t < n to a slot,
// each collision's primaries in order of laser phase (collisions too small
// to sort keep slot order).  Returns false if the batch keeps slot order.
static bool order_collisions(ptg_ctx* c, const double* rows, size_t n_coll, const ptg_collision* coll,
                             const unsigned long long* off, unsigned long long n) {
    bool any = false;
    for (size_t k = 0; k < n_coll; ++k) any = any || coll[k].count >= WAVE_ORDER_MIN;
    if (!any || n > 0xffffffffull || !ensure_order(c, n)) return false;
    k_iota<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(c->d_order, n);
    for (size_t k = 0; k < n_coll; ++k) {
        if (coll[k].count < WAVE_ORDER_MIN) continue;
        if (!order_range(c, WaveKeys{Store{}, rows}, coll[k].first, coll[k].first + coll[k].count,
                         c->d_order + off[k], off[k])) {
            // that collision keeps slot order
            k_iota<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(c->d_order, n);
            return false;
        }
    }
    return cudaGetLastError() == cudaSuccess;
}

// The counting sort of [lo, hi) into out[0, hi - lo) = base + offset.
static bool order_range(ptg_ctx* c, const WaveKeys& s, unsigned long long lo, unsigned long long hi,
                        unsigned long long* out, unsigned long long base) {
    unsigned long long n = hi - lo;
    if (!c->d_buckets) {
        if (cudaMalloc(&c->d_buckets, 4 * WAVE_BUCKETS) != cudaSuccess ||
            cudaMallocHost(&c->h_buckets, 4 * WAVE_BUCKETS) != cudaSuccess ||
            cudaMalloc(&c->d_phase_mm, 16 * WAVE_ORDER_BLOCKS) != cudaSuccess ||
            cudaMallocHost(&c->h_phase_mm, 16 * WAVE_ORDER_BLOCKS) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
    }
    cudaStream_t st = c->stream;
    k_wave_key_range<<<WAVE_ORDER_BLOCKS, 256, 0, st>>>(s, lo, n, c->d_phase_mm);
    if (cudaMemcpyAsync(c->h_phase_mm, c->d_phase_mm, 16 * WAVE_ORDER_BLOCKS, cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return false;
    double mn = HUGE_VAL, mx = -HUGE_VAL;
    for (int b = 0; b < WAVE_ORDER_BLOCKS; ++b) mn = std::min(mn, c->h_phase_mm[2 * b]), mx = std::max(mx, c->h_phase_mm[2 * b + 1]);
    if (!(mx > mn) || !std::isfinite(mx - mn)) return false;
    double inv_width = (double)WAVE_BUCKETS / (mx - mn);
    unsigned blocks = (unsigned)((n + 255) / 256);
    cudaMemsetAsync(c->d_buckets, 0, 4 * WAVE_BUCKETS, st);
    k_wave_bucket_count<<<blocks, 256, 0, st>>>(s, lo, n, mn, inv_width, c->d_buckets);
    if (cudaMemcpyAsync(c->h_buckets, c->d_buckets, 4 * WAVE_BUCKETS, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return false;
    unsigned acc = 0;
    for (int b = 0; b < WAVE_BUCKETS; ++b) {
        unsigned v = c->h_buckets[b];
        c->h_buckets[b] = acc;
        acc += v;
    }
    cudaMemcpyAsync(c->d_buckets, c->h_buckets, 4 * WAVE_BUCKETS, cudaMemcpyHostToDevice, st);
    k_wave_bucket_scatter<<<blocks, 256, 0, st>>>(s, lo, n, mn, inv_width, c->d_buckets, out, base);
    return cudaGetLastError() == cudaSuccess;
}

// Runs a batch whose primaries are described by device pointers `d_in`.
static ptg_status run_batch(ptg_ctx* c, const ptg_laser_desc* laser, const ptg_collide_options* o,
                            const ptg_particles* d_in, uint64_t seed, uint64_t id_base, ptg_run_stats* stats) {
    ptg_status st = check_run(c, laser, o);
    if (st != PTG_OK) return st;
    if (d_in && d_in->n == 0) {
        // no primaries: an empty shower, as collide() mapped over none
        c->d_out.n = 0;
        if (stats) std::memset(stats, 0, sizeof(*stats));
        return PTG_OK;
    }
    if (!d_in || !d_in->species || !d_in->r || !d_in->u)
        return set_err(PTG_ERR_INVALID_ARGUMENT, "primaries need species, r and u");
    bool lcfa = laser->model == PTG_FAST_PLANE_WAVE || laser->model == PTG_FAST_FOCUSED_LASER;
    CUDA_TRY(cudaSetDevice(c->device));
    unsigned long long n = d_in->n;
    double dt_max;
    FieldParams f = make_field(*laser, &dt_max);
    WaveArgs a{};
    a.f = f;
    fill_step_options(*o, &a.o);
    apply_limits(c, &a.o);
    a.o.dt = dt_max * o->dt_multiplier;
    a.gl = c->gl;
    a.lma = c->lma_dev;
    a.mlp = mlp_params(c);
    a.dbw = nullptr;
    a.db_cap = 0;
    c->grid_cap = 0;
    if (!lcfa && laser->polarization != PTG_POL_CIRCULAR) {
        st = ensure_dbw(c, laser->a0, grid_for(c, wave_kernel(laser->model)), &a, &c->grid_cap);
        if (st != PTG_OK) return st;
    }
    a.seed = seed;
    a.n_primaries = n;
    a.id_base = id_base;
    unsigned long long want = c->cap;
    if (want < 8 * n + 1024) want = 8 * n + 1024;
    st = ensure_init(c, n > 0 ? n : 1);
    if (st != PTG_OK) return st;
    CUDA_TRY(cudaEventRecord(c->ev0, c->stream));
    for (int attempt = 0; attempt < 8; ++attempt) {
        st = ensure_store(c, want);
        if (st != PTG_OK) return st;
        a.s = c->s;
        a.c = c->counters;
        CUDA_TRY(cudaMemsetAsync(c->counters, 0, sizeof(Counters), c->stream));
        unsigned long long nt = n;
        CUDA_TRY(cudaMemcpyAsync(&c->counters->n_total, &nt, 8, cudaMemcpyHostToDevice, c->stream));
        if (n > 0) {
            k_load_primaries<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(c->s, *d_in, n, id_base, c->init_u,
                                                                                c->shower_count);
            CUDA_TRY(cudaGetLastError());
        }
        unsigned long long lo = 0, hi = n;
        uint32_t waves = 0, ordered = 0;
        bool overflow = false;
        double wave_ms[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        while (lo < hi) {
            a.lo = lo;
            a.hi = hi;
            a.order = order_wave(c, WaveKeys{c->s, nullptr}, lo, hi) ? c->d_order : nullptr;
            a.warp_batch = (a.order != nullptr && c->warp_batch) ? 1 : 0;
            ordered += a.order ? 1u : 0u;
            CUDA_TRY(cudaMemsetAsync(&c->counters->next, 0, 8, c->stream));
            CUDA_TRY(cudaEventRecord(c->ev_wa, c->stream));
            CUDA_TRY(launch_wave_model(c, a));
            CUDA_TRY(cudaEventRecord(c->ev_wb, c->stream));
            CUDA_TRY(cudaMemcpyAsync(c->h_counters, c->counters, sizeof(Counters), cudaMemcpyDeviceToHost, c->stream));
            CUDA_TRY(cudaStreamSynchronize(c->stream));
            float wms = 0.0f;
            CUDA_TRY(cudaEventElapsedTime(&wms, c->ev_wa, c->ev_wb));
            wave_ms[waves < 8 ? waves : 7] += wms;
            ++waves;
            if (c->h_counters->overflow) {
                overflow = true;
                break;
            }
            lo = hi;
            hi = c->h_counters->n_total;
        }
        if (overflow) {
            // deterministic streams: rerunning with a larger store gives the same shower
            want = 2 * (c->h_counters->n_total > want ? c->h_counters->n_total : want);
            continue;
        }
        unsigned long long total = hi;
        st = ensure_out(c, total > 0 ? total : 1);
        if (st != PTG_OK) return st;
        FilterArgs fa{};
        fa.s = c->s;
        fa.init_u = c->init_u;
        fa.shower_count = c->shower_count;
        fa.n = total;
        fa.min_energy = o->min_energy;
        fa.cos_max_angle = std::cos(o->max_angle);
        fa.discard_bg_e = o->discard_bg_e;
        fa.discard_bg_ph = o->discard_bg_ph;
        fa.multiplicity = o->multiplicity;
        unsigned blocks = (unsigned)((total + 255) / 256);
        if (blocks == 0) blocks = 1;
        if (o->multiplicity >= 0) {
            k_filter_count<<<blocks, 256, 0, c->stream>>>(fa);
            CUDA_TRY(cudaGetLastError());
        }
        k_compact<<<blocks, 256, 0, c->stream>>>(fa, c->counters, c->d_out, c->out_cap);
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaEventRecord(c->ev1, c->stream));
        CUDA_TRY(cudaMemcpyAsync(c->h_counters, c->counters, sizeof(Counters), cudaMemcpyDeviceToHost, c->stream));
        CUDA_TRY(cudaStreamSynchronize(c->stream));
        c->d_out.n = c->h_counters->n_out;
        if (stats) {
            std::memset(stats, 0, sizeof(*stats));
            stats->n_primaries = n;
            stats->n_out = c->h_counters->n_out;
            stats->n_created = total;
            stats->lepton_steps = c->h_counters->lepton_steps;
            stats->photon_steps = c->h_counters->photon_steps;
            stats->emissions = c->h_counters->emissions;
            stats->pair_events = c->h_counters->pair_events;
            stats->rejections = c->h_counters->rejections;
            stats->particle_errors = c->h_counters->errors;
            stats->waves = waves;
            stats->ordered_waves = ordered;
            stats->max_steps = c->h_counters->max_steps;
            stats->free_steps = c->h_counters->free_steps;
            stats->drift_steps = c->h_counters->drift_steps;
            for (int w = 0; w < 8; ++w) stats->wave_ms[w] = wave_ms[w];
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, c->ev0, c->ev1);
            stats->device_ms = ms;
        }
        return PTG_OK;
    }
    return set_err(PTG_ERR_QUEUE_OVERFLOW, "shower store kept overflowing");
}

ptg_status ptg_collide_batch_device(ptg_ctx* c, const ptg_laser_desc* laser, const ptg_collide_options* o,
                                    const ptg_particles* d_primaries, uint64_t seed, uint64_t id_base,
                                    ptg_particles* d_out, ptg_run_stats* stats) {
    if (!c) return set_err(PTG_ERR_INVALID_ARGUMENT, "ctx is NULL");
    ptg_status st = run_batch(c, laser, o, d_primaries, seed, id_base, stats);
    if (st != PTG_OK) return st;
    if (d_out) *d_out = c->d_out;
    return PTG_OK;
}

static ptg_status stage_primaries(ptg_ctx* c, const ptg_particles* h) {
    unsigned long long n = h->n;
    if (n > c->in_cap) {
        if (c->in_mem) cudaFree(c->in_mem);
        c->in_mem = nullptr;
        c->in_cap = 0;
        CUDA_TRY(cudaMalloc(&c->in_mem, particles_bytes(n)));
        carve_particles(&c->d_in, c->in_mem, n);
        c->in_cap = n;
    }
    ptg_particles d = c->d_in;
    d.n = n;
    auto up = [&](void* dst, const void* src, size_t bytes) -> bool {
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream) == cudaSuccess;
    };
    if (n == 0) {
        c->d_in.n = 0;
        return PTG_OK;
    }
    if (!h->species || !h->r || !h->u) return set_err(PTG_ERR_INVALID_ARGUMENT, "primaries need species, r and u");
    bool ok = up(d.species, h->species, 4 * n) && up(d.r, h->r, 32 * n) && up(d.u, h->u, 32 * n);
    if (h->r0) ok = ok && up(d.r0, h->r0, 32 * n); else d.r0 = nullptr;
    if (h->u0) ok = ok && up(d.u0, h->u0, 32 * n); else d.u0 = nullptr;
    if (h->pol) ok = ok && up(d.pol, h->pol, 32 * n); else d.pol = nullptr;
    if (h->weight) ok = ok && up(d.weight, h->weight, 8 * n); else d.weight = nullptr;
    if (h->id) ok = ok && up(d.id, h->id, 8 * n); else d.id = nullptr;
    if (h->parent_id) ok = ok && up(d.parent_id, h->parent_id, 8 * n); else d.parent_id = nullptr;
    if (!ok) return set_err(PTG_ERR_CUDA, "host-to-device copy of the primaries failed");
    c->d_in = d;
    c->d_in.r0 = d.r0, c->d_in.u0 = d.u0;
    return PTG_OK;
}

// ------------------------------------------------ host output blocks ---
// The host arrays of an output live in one page-locked block, so that the
// device-to-host copies run at the link's speed and the pages are not
// faulted in on every call.  A block lent to the caller is recorded here by
// its base (the `r` array) and comes back through ptg_particles_free; the
// context keeps up to two returned blocks for its next outputs and frees
// them when it is destroyed.  A block returned after its context is gone is
// freed at once.
struct HostBlock {
    void* base;
    size_t bytes;
    ptg_ctx* owner;
};
static std::mutex g_host_mu;
static std::unordered_map<void*, HostBlock>& host_lent() {
    static auto* m = new std::unordered_map<void*, HostBlock>();
    return *m;
}
static std::unordered_map<ptg_ctx*, std::vector<HostBlock>>& host_idle() {
    static auto* m = new std::unordered_map<ptg_ctx*, std::vector<HostBlock>>();
    return *m;
}
constexpr size_t HOST_IDLE_MAX = 2;

// A block of at least `bytes` for context c: a returned one if it is large
// enough, else a new one.
static void* host_block_take(ptg_ctx* c, size_t bytes) {
    std::lock_guard<std::mutex> g(g_host_mu);
    auto& idle = host_idle()[c];
    for (size_t k = 0; k < idle.size(); ++k) {
        if (idle[k].bytes >= bytes) {
            HostBlock b = idle[k];
            idle.erase(idle.begin() + (long)k);
            host_lent()[b.base] = b;
            return b.base;
        }
    }
    // room for 12.5 % more particles next time
    size_t want = bytes + bytes / 8;
    void* p = nullptr;
    if (cudaHostAlloc(&p, want, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    host_lent()[p] = HostBlock{p, want, c};
    return p;
}

// Returns true if `base` was a lent block (now given back).
static bool host_block_return(void* base) {
    std::lock_guard<std::mutex> g(g_host_mu);
    auto it = host_lent().find(base);
    if (it == host_lent().end()) return false;
    HostBlock b = it->second;
    host_lent().erase(it);
    if (b.owner == nullptr) {
        cudaFreeHost(b.base);
        return true;
    }
    auto& idle = host_idle()[b.owner];
    idle.push_back(b);
    if (idle.size() > HOST_IDLE_MAX) {
        // drop the smallest
        size_t k_min = 0;
        for (size_t k = 1; k < idle.size(); ++k)
            if (idle[k].bytes < idle[k_min].bytes) k_min = k;
        cudaFreeHost(idle[k_min].base);
        idle.erase(idle.begin() + (long)k_min);
    }
    return true;
}

// The context's returned blocks are freed; its lent ones are freed when
// they come back.
static void host_blocks_release(ptg_ctx* c) {
    std::lock_guard<std::mutex> g(g_host_mu);
    auto it = host_idle().find(c);
    if (it != host_idle().end()) {
        for (auto& b : it->second) cudaFreeHost(b.base);
        host_idle().erase(it);
    }
    for (auto& kv : host_lent())
        if (kv.second.owner == c) kv.second.owner = nullptr;
}

// Copies the context's device output (c->d_out, c->d_out.n rows) into host
// arrays carved from one page-locked block (returned by
// ptg_particles_free); the copies are queued on the context's stream and
// not waited for.
static ptg_status download_output(ptg_ctx* c, ptg_particles* out) {
    size_t m = c->d_out.n;
    std::memset(out, 0, sizeof(*out));
    size_t sz = m ? m : 1;
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    // 8-byte fields first; r is the block's base
    size_t w32 = up(32 * sz), w8 = up(8 * sz), w4 = up(4 * sz);
    size_t bytes = 5 * w32 + 9 * w8 + 4 * w4;
    char* base = (char*)host_block_take(c, bytes);
    if (!base) return set_err(PTG_ERR_ALLOC, "host allocation of the output failed");
    char* q = base;
    auto take = [&](size_t w) {
        char* r = q;
        q += w;
        return r;
    };
    out->r = (double*)take(w32);
    out->u = (double*)take(w32);
    out->r0 = (double*)take(w32);
    out->u0 = (double*)take(w32);
    out->pol = (double*)take(w32);
    out->weight = (double*)take(w8);
    out->payload = (double*)take(w8);
    out->parent_chi = (double*)take(w8);
    out->interaction_count = (double*)take(w8);
    out->work = (double*)take(w8);
    out->id = (uint64_t*)take(w8);
    out->parent_id = (uint64_t*)take(w8);
    out->primary = (uint64_t*)take(w8);
    out->stream = (uint64_t*)take(w8);
    out->species = (int32_t*)take(w4);
    out->generation = (int32_t*)take(w4);
    out->flags = (int32_t*)take(w4);
    out->status = (int32_t*)take(w4);
    out->n = m;
    const ptg_particles& d = c->d_out;
    auto down = [&](void* dst, const void* src, size_t bytes) {
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream);
    };
    if (m) {
        CUDA_TRY(down(out->species, d.species, 4 * m));
        CUDA_TRY(down(out->r, d.r, 32 * m));
        CUDA_TRY(down(out->u, d.u, 32 * m));
        CUDA_TRY(down(out->r0, d.r0, 32 * m));
        CUDA_TRY(down(out->u0, d.u0, 32 * m));
        CUDA_TRY(down(out->pol, d.pol, 32 * m));
        CUDA_TRY(down(out->weight, d.weight, 8 * m));
        CUDA_TRY(down(out->payload, d.payload, 8 * m));
        CUDA_TRY(down(out->parent_chi, d.parent_chi, 8 * m));
        CUDA_TRY(down(out->interaction_count, d.interaction_count, 8 * m));
        CUDA_TRY(down(out->work, d.work, 8 * m));
        CUDA_TRY(down(out->id, d.id, 8 * m));
        CUDA_TRY(down(out->parent_id, d.parent_id, 8 * m));
        CUDA_TRY(down(out->primary, d.primary, 8 * m));
        CUDA_TRY(down(out->stream, d.stream, 8 * m));
        CUDA_TRY(down(out->generation, d.generation, 4 * m));
        CUDA_TRY(down(out->flags, d.flags, 4 * m));
        CUDA_TRY(down(out->status, d.status, 4 * m));
    }
    return PTG_OK;
}

ptg_status ptg_collide_batch(ptg_ctx* c, const ptg_laser_desc* laser, const ptg_collide_options* o,
                             const ptg_particles* primaries, uint64_t seed, uint64_t id_base, ptg_particles* out,
                             ptg_run_stats* stats) {
    if (!c || !primaries || !out) return set_err(PTG_ERR_INVALID_ARGUMENT, "NULL argument");
    CUDA_TRY(cudaSetDevice(c->device));
    ptg_status st = stage_primaries(c, primaries);
    if (st != PTG_OK) return st;
    ptg_particles din = c->d_in;
    // restore carved pointers for the next staging (optional fields may be NULL now)
    carve_particles(&c->d_in, c->in_mem, c->in_cap);
    st = run_batch(c, laser, o, &din, seed, id_base, stats);
    if (st != PTG_OK) return st;
    st = download_output(c, out);
    if (st != PTG_OK) return st;
    size_t m = c->d_out.n;
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (stats) {
        double sum = 0.0;
        for (size_t i = 0; i < m; ++i) sum += out->work[i];
        stats->absorbed_energy = sum * ELECTRON_MASS_MEV;
    }
    return PTG_OK;
}


// ------------------------------------------------ multi-collision queue ---
// Slot i of a multi batch belongs to collision c with off[c] <= i < off[c+1];
// its source row is first[c] + (i - off[c]).
__device__ __forceinline__ int coll_of(const unsigned long long* off, int n_coll, unsigned long long i) {
    int lo = 0, hi = n_coll;  // off[lo] <= i < off[hi]
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (off[mid] <= i)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

__global__ void k_queue_reset(Counters* c, CollStats* st, int n_coll, unsigned long long n) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0) {
        *c = Counters{};
        c->n_total = n;
    }
    if (t < n_coll) st[t] = CollStats{};
}

__global__ void k_load_multi(Store s, ptg_particles in, unsigned long long n, const unsigned long long* off,
                             const unsigned long long* first, const CollParams* cp, int n_coll, double* init_u,
                             unsigned long long* shower_count) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c = coll_of(off, n_coll, i);
    unsigned long long loc = i - off[c];
    load_primary(s, in, first[c] + loc, i, loc, primary_stream(cp[c].id_base + loc), init_u, shower_count);
    s.coll[i] = c;
    s.ready[i] = 1u;
}

// Per-collision output counts and created secondaries; warp-aggregated over
// lanes of the same collision.
__global__ void k_multi_count(FilterArgs fa, CollStats* st, unsigned long long n_prim) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    bool in = in_range(fa, i);
    int c = in ? fa.s.coll[i] : -1;
    bool keep = in && final_keep(fa, i);
    bool created = in && i >= n_prim;
    unsigned peers = __match_any_sync(0xffffffffu, c);
    unsigned nk = __popc(__ballot_sync(0xffffffffu, keep) & peers);
    unsigned nc = __popc(__ballot_sync(0xffffffffu, created) & peers);
    if (in && (threadIdx.x & 31u) == (unsigned)(__ffs(peers) - 1)) {
        if (nk) atomicAdd(&st[c].n_out, (unsigned long long)nk);
        if (nc) atomicAdd(&st[c].n_created, (unsigned long long)nc);
    }
}

__global__ void k_multi_scan(CollStats* st, int n_coll, unsigned long long* out_off, unsigned long long* cursor,
                             Counters* c) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    unsigned long long acc = 0;
    for (int k = 0; k < n_coll; ++k) {
        out_off[k] = acc;
        cursor[k] = acc;
        acc += st[k].n_out;
    }
    out_off[n_coll] = acc;
    c->n_out = acc;
}

__global__ void k_multi_compact(FilterArgs fa, unsigned long long* cursor, ptg_particles o, unsigned long long out_cap) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    bool keep = in_range(fa, i) && final_keep(fa, i);
    int c = keep ? fa.s.coll[i] : -1;
    unsigned peers = __match_any_sync(0xffffffffu, c);
    unsigned keepers = __ballot_sync(0xffffffffu, keep) & peers;
    if (!keep) return;
    unsigned lane = threadIdx.x & 31u;
    unsigned leader = __ffs(keepers) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(&cursor[c], (unsigned long long)__popc(keepers));
    base = __shfl_sync(keepers, base, leader);
    unsigned long long j = base + __popc(keepers & ((1u << lane) - 1u));
    if (j < out_cap) write_row(o, j, fa.s, i);
}

static ptg_status ensure_queue_arrays(ptg_ctx* c, size_t n_coll) {
    if (c->q_cap >= n_coll) return PTG_OK;
    size_t k = std::max<size_t>(n_coll, 64);
    cudaFree(c->d_coll), cudaFree(c->d_cstats), cudaFree(c->d_qoff), cudaFree(c->d_qfirst), cudaFree(c->d_qout),
        cudaFree(c->d_qcursor);
    cudaFreeHost(c->h_coll), cudaFreeHost(c->h_cstats), cudaFreeHost(c->h_qoff), cudaFreeHost(c->h_qfirst),
        cudaFreeHost(c->h_qout);
    c->q_cap = 0;
    if (c->q_graph) {
        cudaGraphExecDestroy(c->q_graph);
        c->q_graph = nullptr;
        c->q_graph_key.clear();
    }
    CUDA_TRY(cudaMalloc(&c->d_coll, sizeof(CollParams) * k));
    CUDA_TRY(cudaMalloc(&c->d_cstats, sizeof(CollStats) * k));
    CUDA_TRY(cudaMalloc(&c->d_qoff, 8 * (k + 1)));
    CUDA_TRY(cudaMalloc(&c->d_qfirst, 8 * k));
    CUDA_TRY(cudaMalloc(&c->d_qout, 8 * (k + 1)));
    CUDA_TRY(cudaMalloc(&c->d_qcursor, 8 * k));
    CUDA_TRY(cudaMallocHost(&c->h_coll, sizeof(CollParams) * k));
    CUDA_TRY(cudaMallocHost(&c->h_cstats, sizeof(CollStats) * k));
    CUDA_TRY(cudaMallocHost(&c->h_qoff, 8 * (k + 1)));
    CUDA_TRY(cudaMallocHost(&c->h_qfirst, 8 * k));
    CUDA_TRY(cudaMallocHost(&c->h_qout, 8 * (k + 1)));
    c->q_cap = k;
    return PTG_OK;
}

static bool lma_model(int model) { return model == M_PLANE_WAVE || model == M_FOCUSED_LASER; }

// The queue kernel of a variant; `model` (an M_* value) selects the
// single-collision kernel's instantiation for variant 2.
static const void* queue_kernel_of(int variant, int model) {
    if (variant == 2) return lma_model(model) ? queue_kernel_single_lma(model) : queue_kernel_single_lcfa(model);
    if (variant == 3) return queue_kernel_v3();
    return variant == 1 ? queue_kernel_v1() : queue_kernel_v0();
}

static cudaError_t launch_queue(int variant, int model, int grid, cudaStream_t s, const QueueArgs& q) {
    if (variant == 2)
        return lma_model(model) ? launch_queue_single_lma(model, grid, s, q) : launch_queue_single_lcfa(model, grid, s, q);
    if (variant == 3) return launch_queue_v3(grid, s, q);
    return variant == 1 ? launch_queue_v1(grid, s, q) : launch_queue_v0(grid, s, q);
}

// Blocks of the queue kernel for a launch shape.
static int queue_grid(ptg_ctx* c, const ptg_queue_cfg& q, int model) {
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, queue_kernel_of(q.variant, model), 128, 0);
    if (occ <= 0) occ = 1;
    int per_sm = q.blocks_per_sm > 0 ? std::min(q.blocks_per_sm, occ) : occ;
    return per_sm * c->num_sms;
}

// The device sequence of one multi batch, on c->stream: reset, load,
// persistent queue kernel, per-collision counts, offsets and compaction,
// and the read-back of the counters into pinned memory.  Captured once per
// shape as a CUDA graph when cfg.use_graph is set.
static cudaError_t enqueue_multi(ptg_ctx* c, const QueueArgs& q, const ptg_particles& d_in, unsigned long long n,
                                 size_t n_coll, int grid, int variant, int model, const FilterArgs& fa_proto,
                                 bool capturing) {
    cudaStream_t s = c->stream;
    cudaError_t e;
    // under capture, external event records become graph nodes that record
    // at replay
    unsigned evf = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
    if ((e = cudaEventRecordWithFlags(c->ev0, s, evf)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(c->d_coll, c->h_coll, sizeof(CollParams) * n_coll, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return e;
    if ((e = cudaMemcpyAsync(c->d_qoff, c->h_qoff, 8 * (n_coll + 1), cudaMemcpyHostToDevice, s)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(c->d_qfirst, c->h_qfirst, 8 * n_coll, cudaMemcpyHostToDevice, s)) != cudaSuccess) return e;
    k_queue_reset<<<(unsigned)((n_coll + 255) / 256) + 1, 256, 0, s>>>(c->counters, c->d_cstats, (int)n_coll, n);
    if ((e = cudaMemsetAsync(c->s.ready, 0, 4 * c->s.cap, s)) != cudaSuccess) return e;
    if (n > 0)
        k_load_multi<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(c->s, d_in, n, c->d_qoff, c->d_qfirst, c->d_coll,
                                                                  (int)n_coll, c->init_u, c->shower_count);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    e = launch_queue(variant, model, grid, s, q);
    if (e != cudaSuccess) return e;
    // compaction over every reserved slot that fits the store (an overflowed
    // batch is rerun, so its output is never read)
    FilterArgs fa = fa_proto;
    fa.n = c->s.cap;
    fa.n_live = &c->counters->n_total;
    unsigned blocks = (unsigned)((c->s.cap + 255) / 256);
    if (fa.multiplicity >= 0) k_filter_count<<<blocks, 256, 0, s>>>(fa);
    k_multi_count<<<blocks, 256, 0, s>>>(fa, c->d_cstats, n);
    k_multi_scan<<<1, 32, 0, s>>>(c->d_cstats, (int)n_coll, c->d_qout, c->d_qcursor, c->counters);
    k_multi_compact<<<blocks, 256, 0, s>>>(fa, c->d_qcursor, c->d_out, c->out_cap);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = cudaEventRecordWithFlags(c->ev1, s, evf)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(c->h_counters, c->counters, sizeof(Counters), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return e;
    if ((e = cudaMemcpyAsync(c->h_cstats, c->d_cstats, sizeof(CollStats) * n_coll, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return e;
    return cudaMemcpyAsync(c->h_qout, c->d_qout, 8 * (n_coll + 1), cudaMemcpyDeviceToHost, s);
}

// Runs a multi batch with device primaries.  On return c->d_out holds the
// output rows (grouped by collision) and c->h_qout their offsets.
static ptg_status run_multi(ptg_ctx* c, size_t n_coll, const ptg_collision* coll, const ptg_collide_options* o,
                            const ptg_particles* d_in, const ptg_queue_cfg& qc, ptg_run_stats* stats,
                            ptg_run_stats* total) {
    if (!c || !coll || !o || !d_in) return set_err(PTG_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n_coll == 0 || n_coll > (1u << 20)) return set_err(PTG_ERR_INVALID_ARGUMENT, "number of collisions out of range");
    if (!d_in->species || !d_in->r || !d_in->u)
        return set_err(PTG_ERR_INVALID_ARGUMENT, "primaries need species, r and u");
    if (qc.variant < 0 || qc.variant > 3 || qc.chunk < 1 || qc.chunk > 64 || qc.blocks_per_sm < 0)
        return set_err(PTG_ERR_INVALID_ARGUMENT, "queue launch shape out of range");
    CUDA_TRY(cudaSetDevice(c->device));
    cudaGetLastError();  // no stale error may reach the capture below
    double lp_lma_a0 = 0.0;
    bool any_lp_lma = false;
    unsigned long long n = 0;
    for (size_t k = 0; k < n_coll; ++k) {
        ptg_status st = check_run(c, &coll[k].laser, o);
        if (st != PTG_OK) return set_err(st, "collision " + std::to_string(k) + ": " + g_last_error);
        if (coll[k].first + coll[k].count > d_in->n || coll[k].first + coll[k].count < coll[k].first)
            return set_err(PTG_ERR_INVALID_ARGUMENT, "collision " + std::to_string(k) + " reads past the primaries");
        bool lcfa = coll[k].laser.model == PTG_FAST_PLANE_WAVE || coll[k].laser.model == PTG_FAST_FOCUSED_LASER;
        if (!lcfa && coll[k].laser.polarization != PTG_POL_CIRCULAR) {
            any_lp_lma = true;
            lp_lma_a0 = std::max(lp_lma_a0, coll[k].laser.a0);
        }
        n += coll[k].count;
    }
    ptg_status st = ensure_queue_arrays(c, n_coll);
    if (st != PTG_OK) return st;
    st = ensure_init(c, n > 0 ? n : 1);
    if (st != PTG_OK) return st;
    // per-collision parameters into the pinned mirrors (read by the copies
    // at the head of the sequence)
    c->h_qoff[0] = 0;
    for (size_t k = 0; k < n_coll; ++k) {
        double dt_max;
        CollParams& cp = c->h_coll[k];
        cp = CollParams{};
        cp.f = make_field(coll[k].laser, &dt_max);
        cp.dt = dt_max * o->dt_multiplier;
        cp.seed = coll[k].seed;
        cp.id_base = coll[k].id_base;
        c->h_qfirst[k] = coll[k].first;
        c->h_qoff[k + 1] = c->h_qoff[k] + coll[k].count;
    }
    // the single-collision kernel runs batches of one collision, with that
    // collision's parameters in its launch arguments; larger batches run
    // variant 0 instead
    int model = c->h_coll[0].f.model;
    int variant = (qc.variant == 2 && n_coll != 1) ? 0 : qc.variant;
    ptg_queue_cfg qe = qc;
    qe.variant = variant;
    int grid = queue_grid(c, qe, model);
    QueueArgs q{};
    if (variant == 2) {
        q.base.f = c->h_coll[0].f;
        q.base.seed = c->h_coll[0].seed;
        q.base.id_base = c->h_coll[0].id_base;
    }
    // primaries in order of laser phase within each collision, from the
    // input rows (before the captured sequence loads them)
    q.base.order = order_collisions(c, d_in->r, n_coll, coll, c->h_qoff, n) ? c->d_order : nullptr;
    fill_step_options(*o, &q.base.o);
    apply_limits(c, &q.base.o);
    if (variant == 2) q.base.o.dt = c->h_coll[0].dt;
    q.base.gl = c->gl;
    q.base.lma = c->lma_dev;
    q.base.mlp = mlp_params(c);
    q.base.n_primaries = n;
    q.coll = c->d_coll;
    q.stats = c->d_cstats;
    q.n_coll = (int)n_coll;
    q.chunk = qc.chunk;
    q.warp_batch = ((variant == 2 || variant == 3) && q.base.order != nullptr && c->warp_batch) ? 1 : 0;
    // longest wait any lane may legitimately see: the drain of the batch's
    // last showers; generous, but bounded
    q.wait_ns = (unsigned long long)(20.0e9 + 2.0e3 * (double)n);
    if (c->limits.queue_wait_ns) q.wait_ns = c->limits.queue_wait_ns;
    if (any_lp_lma) {
        st = ensure_dbw(c, lp_lma_a0, grid, &q.base, &grid);
        if (st != PTG_OK) return st;
    }
    unsigned long long want = c->cap;
    if (want < 4 * n + 1024) want = 4 * n + 1024;
    for (int attempt = 0; attempt < 8; ++attempt) {
        st = ensure_store(c, want);
        if (st != PTG_OK) return st;
        st = ensure_out(c, c->cap);
        if (st != PTG_OK) return st;
        q.base.s = c->s;
        q.base.c = c->counters;
        FilterArgs fa{};
        fa.s = c->s;
        fa.init_u = c->init_u;
        fa.shower_count = c->shower_count;
        fa.min_energy = o->min_energy;
        fa.cos_max_angle = std::cos(o->max_angle);
        fa.discard_bg_e = o->discard_bg_e;
        fa.discard_bg_ph = o->discard_bg_ph;
        fa.multiplicity = o->multiplicity;
        if (qc.use_graph) {
            char key[512];
            std::snprintf(key, sizeof key, "%llu/%zu/%llu/%llu/%d/%d/%d/%p/%p/%p/%p/%p/%p/%p/%p/%d/%p/%d", n, n_coll,
                          c->s.cap, c->out_cap, grid, variant * 8 + (model + 1) + (q.base.order ? 64 : 0), qc.chunk,
                          (void*)d_in->species, (void*)d_in->r,
                          (void*)d_in->u, (void*)d_in->pol, (void*)d_in->weight, (void*)d_in->id, (void*)d_in->r0,
                          (void*)d_in->u0, q.base.db_cap, (void*)q.base.dbw, (int)sizeof(StepOptions));
            std::string k = key;
            // the kernel's arguments are captured by value: every byte of them
            // (the single-collision kernel's laser, seed and id base, the
            // learned proposal's switch and margin, the step options, the
            // phase order) must match for a replay
            k.append((const char*)&q, sizeof(q));
            k.append((const char*)&fa.min_energy, 2 * sizeof(double));
            k.append((const char*)&fa.discard_bg_e, 3 * sizeof(int));
            if (!c->q_graph || k != c->q_graph_key) {
                if (c->q_graph) cudaGraphExecDestroy(c->q_graph);
                c->q_graph = nullptr;
                c->q_graph_key.clear();
                cudaGraph_t g = nullptr;
                CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
                cudaError_t e = enqueue_multi(c, q, *d_in, n, n_coll, grid, variant, model, fa, true);
                cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
                if (e != cudaSuccess || e2 != cudaSuccess) {
                    if (g) cudaGraphDestroy(g);
                    cudaGetLastError();
                    return set_err(PTG_ERR_CUDA, std::string("graph capture of the queue batch: ") +
                                                     cudaGetErrorString(e != cudaSuccess ? e : e2));
                }
                cudaError_t e3 = cudaGraphInstantiate(&c->q_graph, g, 0);
                cudaGraphDestroy(g);
                if (e3 != cudaSuccess) {
                    c->q_graph = nullptr;
                    return set_err(PTG_ERR_CUDA, std::string("graph instantiation: ") + cudaGetErrorString(e3));
                }
                c->q_graph_key = k;
            }
            CUDA_TRY(cudaGraphLaunch(c->q_graph, c->stream));
        } else {
            CUDA_TRY(enqueue_multi(c, q, *d_in, n, n_coll, grid, variant, model, fa, false));
        }
        CUDA_TRY(cudaStreamSynchronize(c->stream));
        const Counters& h = *c->h_counters;
        if (h.overflow) {
            want = 2 * (h.n_total > want ? h.n_total : want);
            continue;
        }
        if (h.timeouts) return set_err(PTG_ERR_TIMEOUT, "queue kernel: a bounded wait ran out");
        if (h.completed != h.n_total)
            return set_err(PTG_ERR_TIMEOUT, "queue kernel finished with " + std::to_string(h.n_total - h.completed) +
                                                " slots unprocessed");
        c->d_out.n = h.n_out;
        float ms = 0.0f;
        CUDA_TRY(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
        if (total) std::memset(total, 0, sizeof(*total));
        for (size_t k = 0; k < n_coll; ++k) {
            const CollStats& cs = c->h_cstats[k];
            ptg_run_stats r{};
            r.n_primaries = coll[k].count;
            r.n_out = cs.n_out;
            r.n_created = coll[k].count + cs.n_created;
            r.lepton_steps = cs.lepton_steps;
            r.photon_steps = cs.photon_steps;
            r.free_steps = cs.free_steps;
            r.drift_steps = cs.drift_steps;
            r.emissions = cs.emissions;
            r.pair_events = cs.pair_events;
            r.rejections = cs.rejections;
            r.particle_errors = cs.errors;
            r.waves = (uint32_t)(attempt + 1);  // queue launches, reruns after an overflow included
            r.device_ms = ms;
            if (stats) stats[k] = r;
            if (total) {
                total->n_primaries += r.n_primaries;
                total->n_out += r.n_out;
                total->n_created += r.n_created;
                total->lepton_steps += r.lepton_steps;
                total->photon_steps += r.photon_steps;
                total->free_steps += r.free_steps;
                total->drift_steps += r.drift_steps;
                total->emissions += r.emissions;
                total->pair_events += r.pair_events;
                total->rejections += r.rejections;
                total->particle_errors += r.particle_errors;
            }
        }
        if (total) {
            total->particle_errors += h.errors;
            total->waves = (uint32_t)(attempt + 1);
            total->max_steps = h.max_steps;
            total->device_ms = ms;
        }
        return PTG_OK;
    }
    return set_err(PTG_ERR_QUEUE_OVERFLOW, "shower store kept overflowing");
}

ptg_status ptg_collide_multi_device(ptg_ctx* c, size_t n_coll, const ptg_collision* coll,
                                    const ptg_collide_options* o, const ptg_particles* d_primaries,
                                    ptg_particles* d_out, uint64_t* out_offsets, ptg_run_stats* stats,
                                    ptg_run_stats* total) {
    if (!c) return set_err(PTG_ERR_INVALID_ARGUMENT, "ctx is NULL");
    ptg_status st = run_multi(c, n_coll, coll, o, d_primaries, c->qcfg, stats, total);
    if (st != PTG_OK) return st;
    if (d_out) *d_out = c->d_out;
    if (out_offsets)
        for (size_t k = 0; k <= n_coll; ++k) out_offsets[k] = c->h_qout[k];
    return PTG_OK;
}

ptg_status ptg_collide_multi(ptg_ctx* c, size_t n_coll, const ptg_collision* coll, const ptg_collide_options* o,
                             const ptg_particles* primaries, ptg_particles* out, uint64_t* out_offsets,
                             ptg_run_stats* stats, ptg_run_stats* total) {
    if (!c || !primaries || !out) return set_err(PTG_ERR_INVALID_ARGUMENT, "NULL argument");
    CUDA_TRY(cudaSetDevice(c->device));
    ptg_status st = stage_primaries(c, primaries);
    if (st != PTG_OK) return st;
    ptg_particles din = c->d_in;
    carve_particles(&c->d_in, c->in_mem, c->in_cap);
    st = run_multi(c, n_coll, coll, o, &din, c->qcfg, stats, total);
    if (st != PTG_OK) return st;
    st = download_output(c, out);
    if (st != PTG_OK) return st;
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (out_offsets)
        for (size_t k = 0; k <= n_coll; ++k) out_offsets[k] = c->h_qout[k];
    // absorbed energy per collision, from the downloaded work column
    for (size_t k = 0; k < n_coll; ++k) {
        double sum = 0.0;
        for (uint64_t i = c->h_qout[k]; i < c->h_qout[k + 1]; ++i) sum += out->work[i];
        if (stats) stats[k].absorbed_energy = sum * ELECTRON_MASS_MEV;
        if (total) total->absorbed_energy += sum * ELECTRON_MASS_MEV;
    }
    return PTG_OK;
}

ptg_status ptg_queue_config(ptg_ctx* c, const ptg_queue_cfg* cfg, ptg_queue_cfg* cfg_out) {
    if (!c) return set_err(PTG_ERR_INVALID_ARGUMENT, "ctx is NULL");
    if (cfg) {
        if (cfg->variant < 0 || cfg->variant > 3 || cfg->chunk < 1 || cfg->chunk > 64 || cfg->blocks_per_sm < 0)
            return set_err(PTG_ERR_INVALID_ARGUMENT, "queue launch shape out of range");
        c->qcfg = *cfg;
    }
    if (cfg_out) *cfg_out = c->qcfg;
    return PTG_OK;
}

// The autotuner: every candidate shape runs the sample batch once to warm
// up (and to size the store), then twice timed with the batch's device
// events; the fastest mean is kept.
ptg_status ptg_queue_autotune(ptg_ctx* c, size_t n_coll, const ptg_collision* coll, const ptg_collide_options* o,
                              const ptg_particles* d_primaries, double sample_fraction, ptg_queue_cfg* best,
                              double* best_ms) {
    if (!c || !coll || !o || !d_primaries) return set_err(PTG_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!(sample_fraction > 0.0 && sample_fraction <= 1.0))
        return set_err(PTG_ERR_INVALID_ARGUMENT, "sample_fraction must lie in (0, 1]");
    CUDA_TRY(cudaSetDevice(c->device));
    // a single collision's sample fills every lane the kernel can hold twice
    // over, so that the shapes are compared at the occupancy they will run
    // at; several collisions run side by side and fill the device together
    uint64_t floor_count = n_coll == 1 ? 2ull * (uint64_t)c->num_sms * 3ull * 128ull : 1ull;
    std::vector<ptg_collision> sample(coll, coll + n_coll);
    for (auto& s : sample) {
        uint64_t m = (uint64_t)std::ceil(sample_fraction * (double)s.count);
        s.count = std::min<uint64_t>(s.count, std::max<uint64_t>(m, floor_count));
    }
    // the single-collision variant is a candidate for a batch of one, the
    // lockstep multi-collision variant for larger batches
    double dt_max;
    int model = make_field(coll[0].laser, &dt_max).model;
    std::vector<int> vars = n_coll == 1 ? std::vector<int>{0, 1, 2} : std::vector<int>{0, 1, 3};
    std::vector<ptg_queue_cfg> cands;
    for (int v : vars) {
        int occ = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, queue_kernel_of(v, model), 128, 0);
        if (occ < 1) occ = 1;
        for (int bps : {occ, occ > 1 ? occ - 1 : 0})
            for (int chunk : {1, 2})
                if (bps > 0) cands.push_back(ptg_queue_cfg{v, bps, chunk, 1});
    }
    double best_t = 1e300;
    ptg_queue_cfg best_c = c->qcfg;
    for (const auto& cand : cands) {
        ptg_status st = run_multi(c, n_coll, sample.data(), o, d_primaries, cand, nullptr, nullptr);
        if (st != PTG_OK) return st;
        double t = 0.0;
        for (int rep = 0; rep < 2; ++rep) {
            ptg_run_stats tot{};
            st = run_multi(c, n_coll, sample.data(), o, d_primaries, cand, nullptr, &tot);
            if (st != PTG_OK) return st;
            t += tot.device_ms;
        }
        t *= 0.5;
        if (t < best_t) {
            best_t = t;
            best_c = cand;
        }
    }
    c->qcfg = best_c;
    if (best) *best = best_c;
    if (best_ms) *best_ms = best_t;
    return PTG_OK;
}

void ptg_particles_free(ptg_particles* p) {
    if (!p) return;
    if (p->r && host_block_return(p->r)) {
        std::memset(p, 0, sizeof(*p));
        return;
    }
    std::free(p->species);
    std::free(p->r);
    std::free(p->u);
    std::free(p->r0);
    std::free(p->u0);
    std::free(p->pol);
    std::free(p->weight);
    std::free(p->payload);
    std::free(p->parent_chi);
    std::free(p->interaction_count);
    std::free(p->work);
    std::free(p->id);
    std::free(p->parent_id);
    std::free(p->primary);
    std::free(p->stream);
    std::free(p->generation);
    std::free(p->flags);
    std::free(p->status);
    std::memset(p, 0, sizeof(*p));
}

// ---------------------------------------------------- diagnostics ABI ---
template <typename F>
static ptg_status with_device_buffers(ptg_ctx* c, std::vector<std::pair<void*, size_t>> bufs, F f) {
    std::vector<void*> d(bufs.size(), nullptr);
    ptg_status st = PTG_OK;
    for (size_t i = 0; i < bufs.size(); ++i) {
        if (cudaMalloc(&d[i], bufs[i].second ? bufs[i].second : 8) != cudaSuccess) {
            cudaGetLastError();
            st = set_err(PTG_ERR_ALLOC, "diagnostic buffer allocation failed");
            break;
        }
        if (bufs[i].first) cudaMemcpy(d[i], bufs[i].first, bufs[i].second, cudaMemcpyHostToDevice);
    }
    if (st == PTG_OK) {
        f(d);
        cudaError_t e = cudaStreamSynchronize(c->stream);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e != cudaSuccess) st = set_err(PTG_ERR_CUDA, cudaGetErrorString(e));
        for (size_t i = 0; i < bufs.size() && st == PTG_OK; ++i)
            if (bufs[i].first) cudaMemcpy(bufs[i].first, d[i], bufs[i].second, cudaMemcpyDeviceToHost);
    }
    for (void* p : d) cudaFree(p);
    return st;
}

ptg_status ptg_eval_fields(ptg_ctx* c, const ptg_laser_desc* laser, size_t n, const double* r, double* E, double* B,
                           double* a) {
    if (!c) return set_err(PTG_ERR_INVALID_ARGUMENT, "ctx is NULL");
    ptg_status st = check_laser(laser);
    if (st != PTG_OK) return st;
    double dt;
    FieldParams f = make_field(*laser, &dt);
    cudaSetDevice(c->device);
    std::vector<double> rr(r, r + 4 * n);
    return with_device_buffers(c, {{rr.data(), 32 * n}, {E, 24 * n}, {B, 24 * n}, {a, 8 * n}}, [&](std::vector<void*>& d) {
        k_eval_fields<<<(unsigned)((n + 127) / 128) + 1, 128, 0, c->stream>>>(f, n, (double*)d[0], (double*)d[1],
                                                                              (double*)d[2], (double*)d[3]);
    });
}

ptg_status ptg_push_steps(ptg_ctx* c, const ptg_laser_desc* laser, size_t n, double* r, double* u, double rqm,
                          double dt, int32_t eqn, int32_t nsteps, double* work) {
    if (!c) return set_err(PTG_ERR_INVALID_ARGUMENT, "ctx is NULL");
    ptg_status st = check_laser(laser);
    if (st != PTG_OK) return st;
    double dtm;
    FieldParams f = make_field(*laser, &dtm);
    cudaSetDevice(c->device);
    std::vector<double> wk(n, 0.0);
    st = with_device_buffers(c, {{r, 32 * n}, {u, 32 * n}, {wk.data(), 8 * n}}, [&](std::vector<void*>& d) {
        k_push_steps<<<(unsigned)((n + 127) / 128) + 1, 128, 0, c->stream>>>(f, n, (double*)d[0], (double*)d[1], rqm, dt,
                                                                             eqn, nsteps, (double*)d[2]);
    });
    if (st == PTG_OK && work) std::memcpy(work, wk.data(), 8 * n);
    return st;
}

ptg_status ptg_lcfa_photon_rate(ptg_ctx* c, size_t n, const double* chi, const double* gamma, double* rate) {
    if (!c) return set_err(PTG_ERR_INVALID_ARGUMENT, "ctx is NULL");
    cudaSetDevice(c->device);
    std::vector<double> a(chi, chi + n), b(gamma, gamma + n);
    return with_device_buffers(c, {{a.data(), 8 * n}, {b.data(), 8 * n}, {rate, 8 * n}}, [&](std::vector<void*>& d) {
        k_photon_rate<<<(unsigned)((n + 127) / 128) + 1, 128, 0, c->stream>>>(n, (double*)d[0], (double*)d[1], (double*)d[2]);
    });
}

ptg_status ptg_lcfa_photon_sample(ptg_ctx* c, size_t n, const double* chi, const double* gamma, const double* rand3,
                                  double* omega, double* theta) {
    if (!c) return set_err(PTG_ERR_INVALID_ARGUMENT, "ctx is NULL");
    cudaSetDevice(c->device);
    std::vector<double> a(chi, chi + n), b(gamma, gamma + n), r(rand3, rand3 + 3 * n);
    return with_device_buffers(c, {{a.data(), 8 * n}, {b.data(), 8 * n}, {r.data(), 24 * n}, {omega, 8 * n}, {theta, 8 * n}},
                               [&](std::vector<void*>& d) {
                                   k_photon_sample<<<(unsigned)((n + 127) / 128) + 1, 128, 0, c->stream>>>(
                                       n, (double*)d[0], (double*)d[1], (double*)d[2], (double*)d[3], (double*)d[4]);
                               });
}

ptg_status ptg_double_bessel(ptg_ctx* c, int32_t n, size_t count, const double* x, const double* y, int32_t mode,
                             double* j5) {
    if (!c || !x || !y || !j5) return set_err(PTG_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n < 1 || n > 1000000) return set_err(PTG_ERR_INVALID_ARGUMENT, "order out of range");
    if (count == 0) return PTG_OK;
    cudaSetDevice(c->device);
    int cap = db_len_for(n);
    size_t lanes = (count + 31) / 32 * 32;
    std::vector<double> a(x, x + count), b(y, y + count);
    std::vector<int> ok(count, 0);
    ptg_status st = with_device_buffers(
        c, {{a.data(), 8 * count}, {b.data(), 8 * count}, {nullptr, lanes * (size_t)cap * 40}, {j5, 40 * count},
            {ok.data(), 4 * count}},
        [&](std::vector<void*>& d) {
            k_double_bessel<<<(unsigned)((count + 127) / 128), 128, 0, c->stream>>>(
                count, n, cap, (double*)d[0], (double*)d[1], mode, (double*)d[2], (double*)d[3], (int*)d[4]);
        });
    if (st != PTG_OK) return st;
    for (size_t i = 0; i < count; ++i)
        if (!ok[i]) return set_err(PTG_ERR_INVALID_ARGUMENT, "(x, y) outside 0 <= x <= n sqrt 2, 0 <= y <= n / 2");
    return PTG_OK;
}

static ptg_status lp_sample_points(ptg_ctx* c, size_t count, const double* a, const double* eta, uint64_t seed,
                                   const uint64_t* stream, uint32_t step, double* out7, int32_t* status, bool warp) {
    if (!c || !a || !eta || !stream || !out7 || !status) return set_err(PTG_ERR_INVALID_ARGUMENT, "NULL argument");
    if (count == 0) return PTG_OK;
    if (!c->tables_loaded) {
        ptg_status st = ptg_load_tables(c, nullptr);
        if (st != PTG_OK) return st;
    }
    cudaSetDevice(c->device);
    double amax = 0.0;
    for (size_t i = 0; i < count; ++i) amax = std::max(amax, a[i]);
    int n_cap = (int)std::ceil(1.5 * (6.0 * (1.0 + amax * amax) + 2.0 * amax * amax * amax)) + 16;
    int cap = db_len_for(n_cap);
    size_t lanes = (count + 31) / 32 * 32;
    std::vector<double> va(a, a + count), ve(eta, eta + count);
    std::vector<unsigned long long> vs(stream, stream + count);
    return with_device_buffers(
        c, {{va.data(), 8 * count}, {ve.data(), 8 * count}, {vs.data(), 8 * count}, {nullptr, lanes * (size_t)cap * 40},
            {out7, 56 * count}, {status, 4 * count}},
        [&](std::vector<void*>& d) {
            // the workspace holds one slot per lane of ceil(count / 32)
            // warps; k_lp_sample_warp's warps past the last point stop
            // before they touch it
            auto kern = warp ? k_lp_sample_warp : k_lp_sample;
            kern<<<(unsigned)((count + 127) / 128), 128, 0, c->stream>>>(
                count, cap, c->lma_dev, (double*)d[0], (double*)d[1], seed, (unsigned long long*)d[2], step,
                (double*)d[3], (double*)d[4], (int*)d[5]);
        });
}

// One CP harmonic/s/azimuth/Stokes sample per point (cp_sample, or with
// `warp` cp_sample_warp, each warp sampling its 32 points one after another).
__global__ void k_cp_sample(unsigned long long m, int warp, MlpParams mlp, const LmaTables* t, const double* a,
                            const double* eta, unsigned long long seed, const unsigned long long* stream, unsigned step,
                            double* out7, int* status) {
    __shared__ __align__(16) float s_mlp[4][2 * MLP_H];
    if (mlp.enabled && warp) mlp_stage(mlp, mlp_smem());
    unsigned long long base = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) & ~31ull;
    const unsigned lane = threadIdx.x & 31u;
    // warp: point base + q for q = 0..31, every lane together; otherwise
    // point base + lane on its own lane
    for (unsigned q = 0; q < (warp ? 32u : 1u); ++q) {
        unsigned long long i = base + (warp ? q : lane);
        if (i >= m) break;  // with warp, the same for every lane of the warp
        Draws rng;
        rng.begin(seed, stream[i], step);
        int n = 0;
        double s = 0.0, th = 0.0;
        d3 sv = mk3(0.0, 0.0, 0.0);
        uint32_t rej = 0;
        int st;
        if (mlp.enabled)
            st = warp ? cp_sample_learned_warp(*mlp_smem(), mlp, nlc_view(*t), s_mlp[threadIdx.x >> 5], a[i], eta[i],
                                               rng, &n, &s, &th, &sv, &rej)
                      : cp_sample_learned_lane(mlp, nlc_view(*t), a[i], eta[i], rng, &n, &s, &th, &sv, &rej);
        else
            st = warp ? cp_sample_warp(nlc_view(*t), a[i], eta[i], rng, &n, &s, &th, &sv, &rej)
                      : cp_sample(nlc_view(*t), a[i], eta[i], rng, &n, &s, &th, &sv, &rej);
        if (!warp || lane == q) {
            status[i] = st;
            double* o = out7 + 7 * i;
            o[0] = n, o[1] = s, o[2] = th, o[3] = 1.0, o[4] = sv.x, o[5] = sv.y, o[6] = sv.z;
        }
    }
}

static ptg_status cp_sample_points(ptg_ctx* c, size_t count, const double* a, const double* eta, uint64_t seed,
                                   const uint64_t* stream, uint32_t step, double* out7, int32_t* status, bool warp,
                                   bool learned = false) {
    if (!c || !a || !eta || !stream || !out7 || !status) return set_err(PTG_ERR_INVALID_ARGUMENT, "NULL argument");
    if (count == 0) return PTG_OK;
    if (!c->tables_loaded) {
        ptg_status st = ptg_load_tables(c, nullptr);
        if (st != PTG_OK) return st;
    }
    MlpParams mlp{};
    if (learned) {
        mlp = mlp_params(c);
        if (!mlp.enabled) return set_err(PTG_ERR_INVALID_ARGUMENT, "no trained network in use (ptg_mlp_use)");
    }
    cudaSetDevice(c->device);
    std::vector<double> va(a, a + count), ve(eta, eta + count);
    std::vector<unsigned long long> vs(stream, stream + count);
    return with_device_buffers(c, {{va.data(), 8 * count}, {ve.data(), 8 * count}, {vs.data(), 8 * count},
                                   {out7, 56 * count}, {status, 4 * count}},
                               [&](std::vector<void*>& d) {
                                   k_cp_sample<<<(unsigned)((count + 127) / 128), 128, 0, c->stream>>>(
                                       count, warp ? 1 : 0, mlp, c->lma_dev, (double*)d[0], (double*)d[1], seed,
                                       (unsigned long long*)d[2], step, (double*)d[3], (int*)d[4]);
                               });
}

ptg_status ptg_cp_sample(ptg_ctx* c, size_t count, const double* a, const double* eta, uint64_t seed,
                         const uint64_t* stream, uint32_t step, double* out7, int32_t* status) {
    return cp_sample_points(c, count, a, eta, seed, stream, step, out7, status, false);
}

ptg_status ptg_cp_sample_warp(ptg_ctx* c, size_t count, const double* a, const double* eta, uint64_t seed,
                              const uint64_t* stream, uint32_t step, double* out7, int32_t* status) {
    return cp_sample_points(c, count, a, eta, seed, stream, step, out7, status, true);
}

ptg_status ptg_cp_sample_learned(ptg_ctx* c, size_t count, const double* a, const double* eta, uint64_t seed,
                                 const uint64_t* stream, uint32_t step, int32_t warp, double* out7, int32_t* status) {
    return cp_sample_points(c, count, a, eta, seed, stream, step, out7, status, warp != 0, true);
}

ptg_status ptg_lp_sample(ptg_ctx* c, size_t count, const double* a, const double* eta, uint64_t seed,
                         const uint64_t* stream, uint32_t step, double* out7, int32_t* status) {
    return lp_sample_points(c, count, a, eta, seed, stream, step, out7, status, false);
}

ptg_status ptg_lp_sample_warp(ptg_ctx* c, size_t count, const double* a, const double* eta, uint64_t seed,
                              const uint64_t* stream, uint32_t step, double* out7, int32_t* status) {
    return lp_sample_points(c, count, a, eta, seed, stream, step, out7, status, true);
}

ptg_status ptg_lcfa_pair_t(ptg_ctx* c, size_t n, const double* chi, double* t_par, double* t_perp) {
    if (!c) return set_err(PTG_ERR_INVALID_ARGUMENT, "ctx is NULL");
    cudaSetDevice(c->device);
    std::vector<double> a(chi, chi + n);
    return with_device_buffers(c, {{a.data(), 8 * n}, {t_par, 8 * n}, {t_perp, 8 * n}}, [&](std::vector<void*>& d) {
        k_pair_t<<<(unsigned)((n + 127) / 128) + 1, 128, 0, c->stream>>>(n, (double*)d[0], (double*)d[1], (double*)d[2]);
    });
}


// main.rs:294-319 (increase_pair_rate_by, increase_lcfa_pair_rate_by): the
// photon emission probability over the pair creation probability for a
// particle of Lorentz factor gamma meeting the laser head on.  out[0] is the
// ratio, out[1] a ptg status (the lookups the reference unwraps may leave
// their tables).
__global__ void k_pair_rate_increase(int lcfa, int circular, double gamma, double a0, double wavelength,
                                     const LmaTables* lma, double* out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (lcfa) {
        double omega_mc2 = 1.26e-6 / (ELECTRON_MASS_MEV * 1.0e6 * wavelength);
        double chi = 2.0 * gamma * a0 * omega_mc2;
        double t_par, t_perp;
        lcfa_auxiliary_t(chi, &t_par, &t_perp);
        // lcfa::pair_creation::probability for an unpolarised photon, dt = 1
        double pair = ALPHA_FINE * chi * (0.5 * t_par + 0.5 * t_perp) * 1.0 / (COMPTON_TIME * gamma);
        out[0] = lcfa_photon_rate(chi, gamma) / pair;
        out[1] = 0.0;
        return;
    }
    double kk = SPEED_OF_LIGHT * COMPTON_TIME * 2.0 * PI / wavelength;
    d4 kappa = d4{kk, 0.0, 0.0, kk};
    d4 ell = d4{gamma, 0.0, 0.0, -gamma};
    d4 u = d4{sqrt(1.0 + gamma * gamma), 0.0, 0.0, -gamma};
    double a_rms = circular ? a0 : a0 / SQRT_2;
    double sq = a_rms * a_rms / (2.0 * dot4(kappa, u));
    d4 q = d4{u.t + sq * kappa.t, u.x + sq * kappa.x, u.y + sq * kappa.y, u.z + sq * kappa.z};
    double dt = wavelength / SPEED_OF_LIGHT;
    // pair_creation::probability (pair_creation/mod.rs:21-42), unpolarised
    double eta = dot4(kappa, ell);
    double dphi = eta * dt / (COMPTON_TIME * ell.t);
    double f[2] = {0.0, 0.0};
    bool ok = circular ? bw_rates(lma->bw_cp_total, a_rms, eta, &f[0], &f[1])
                       : lpp_rates(lma->bw_lp_total, lma->bw_lp_mid_total, a_rms * SQRT_2, eta, f);
    double pair = (ALPHA_FINE * dphi / eta) * (0.5 * (f[0] + f[1]));
    // nonlinear_compton::probability (nonlinear_compton/mod.rs:19-47)
    double a2 = dot4(q, q) - 1.0;
    double a = a2 >= 0.0 ? sqrt(a2) : 0.0;
    double eta_q = dot4(kappa, q);
    double dphi_q = dt * eta_q / (COMPTON_TIME * q.t);
    double rate = 0.0;
    NlcTables nt = nlc_view(*lma);
    bool ok_q = circular ? cp_rate(nt, a, eta_q, &rate) : lp_rate(nt, a * SQRT_2, eta_q, &rate);
    double photon = ALPHA_FINE * rate * dphi_q / eta_q;
    out[0] = (pair == 0.0) ? 1.0 : fmax(photon / pair, 1.0);
    out[1] = (ok && ok_q) ? 0.0 : 2.0;  // PTG_ERR_OUT_OF_TABLE
}

// The emission step's FP32 rate (emission_rate32) beside the FP64 rate
// (cp_rate / lp_rate) at a^2 = u.u - 1 and eta: out[3 i] the FP32 rate (or
// NaN where it does not apply), out[3 i + 1] the FP64 rate, out[3 i + 2] 1
// if the FP64 rate is in table, else 0.
__global__ void k_emission_rate_pair(unsigned long long n, int circular, const LmaTables* t, const double* a2,
                                     const double* eta, double* out) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float r32 = 0.0f;
    bool in32 = emission_rate32(*t, circular != 0, a2[i], eta[i], &r32);
    double aq = a2[i] >= 0.0 ? sqrt(a2[i]) : 0.0;
    double rate = 0.0;
    NlcTables nt = nlc_view(*t);
    bool ok = circular ? cp_rate(nt, aq, eta[i], &rate) : lp_rate(nt, aq * SQRT_2, eta[i], &rate);
    out[3 * i] = in32 ? (double)r32 : __longlong_as_double(0x7ff8000000000000LL);
    out[3 * i + 1] = rate;
    out[3 * i + 2] = ok ? 1.0 : 0.0;
}

ptg_status ptg_emission_rate_bound(ptg_ctx* c, size_t n, int32_t circular, const double* a_sqd, const double* eta,
                                   double* out3) {
    if (!c || (n && (!a_sqd || !eta || !out3))) return set_err(PTG_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n == 0) return PTG_OK;
    if (!c->tables_loaded) {
        ptg_status st = ptg_load_tables(c, nullptr);
        if (st != PTG_OK) return st;
    }
    CUDA_TRY(cudaSetDevice(c->device));
    std::vector<double> va(a_sqd, a_sqd + n), ve(eta, eta + n);
    return with_device_buffers(c, {{va.data(), 8 * n}, {ve.data(), 8 * n}, {out3, 24 * n}},
                               [&](std::vector<void*>& d) {
                                   k_emission_rate_pair<<<(unsigned)((n + 127) / 128), 128, 0, c->stream>>>(
                                       n, circular ? 1 : 0, c->lma_dev, (double*)d[0], (double*)d[1], (double*)d[2]);
                               });
}

ptg_status ptg_pair_rate_increase(ptg_ctx* c, const ptg_laser_desc* laser, double gamma, double* ratio) {
    if (!c || !ratio) return set_err(PTG_ERR_INVALID_ARGUMENT, "NULL argument");
    ptg_status st = check_laser(laser);
    if (st != PTG_OK) return st;
    if (!(gamma >= 1.0)) return set_err(PTG_ERR_INVALID_ARGUMENT, "gamma must be at least 1");
    bool lcfa = laser->model == PTG_FAST_PLANE_WAVE || laser->model == PTG_FAST_FOCUSED_LASER;
    CUDA_TRY(cudaSetDevice(c->device));
    if (!lcfa && !c->tables_loaded) {
        st = ptg_load_tables(c, nullptr);
        if (st != PTG_OK) return st;
    }
    double out[2] = {0.0, 0.0};
    st = with_device_buffers(c, {{out, sizeof(out)}}, [&](std::vector<void*>& d) {
        k_pair_rate_increase<<<1, 32, 0, c->stream>>>(lcfa ? 1 : 0, laser->polarization == PTG_POL_CIRCULAR ? 1 : 0,
                                                      gamma, laser->a0, laser->wavelength, c->lma_dev, (double*)d[0]);
    });
    if (st != PTG_OK) return st;
    if (out[1] != 0.0) return set_err(PTG_ERR_OUT_OF_TABLE, "a rate lookup left its table");
    *ratio = out[0];
    return PTG_OK;
}

// ------------------------------------------------- table maintenance ---
// Regenerates the CP harmonic CDF table on the device (the reference tree
// lacks nonlinear_compton/cp/tables/cdf.rs; its generator is
// nonlinear_compton/cp/mod.rs:472-612).  Grid: a = 0.02 * 10^(j/20),
// j < 61; eta = 1e-3 * 10^(i/20), i < 70; n_max = 10 (1 + a^3).
namespace ptg {

// -------------------------------------------------- table regeneration --
// The CP harmonic CDF table (nonlinear_compton/cp/tables/cdf.rs) is not in
// the reference tree; its generator is nonlinear_compton/cp/mod.rs:472-612.
// Pass 1: one thread per (grid point, harmonic) computes the partial rate.
struct RegenChunk {
    int point;     // grid point index (eta row * 61 + a column)
    int n0;        // first harmonic of this block
};

__global__ void k_regen_cp_partial(const RegenChunk* chunks, const double* a_of, const double* eta_of,
                                   const int* nmax_of, const unsigned long long* offset_of, double* rates) {
    RegenChunk ch = chunks[blockIdx.x];
    int n = ch.n0 + (int)threadIdx.x;
    if (n > nmax_of[ch.point]) return;
    double a = a_of[ch.point], eta = eta_of[ch.point];
    rates[offset_of[ch.point] + (n - 1)] = cp_partial_rate(n, a, eta);
}

// Pass 2: one thread per grid point: the cumulative sum in harmonic order
// and the 32 CDF nodes of the reference's generator.
__global__ void k_regen_cp_cdf(int npoints, const int* nmax_of, const unsigned long long* offset_of, const double* rates,
                               double* cum /* [sum nmax][2] */, double* cdf_out /* [npoints][32][2] */,
                               double* total_out /* [npoints] */) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npoints) return;
    int n_max = nmax_of[p];
    const double* r = rates + offset_of[p];
    double* c = cum + 2 * offset_of[p];
    double cs = 0.0;
    for (int n = 1; n <= n_max; ++n) {
        cs = cs + r[n - 1];
        c[2 * (n - 1)] = (double)n;
        c[2 * (n - 1) + 1] = cs;
    }
    double rate = cs;
    double* out = cdf_out + (size_t)p * 64;
    out[0] = c[0];
    out[1] = c[1] / rate;
    double limit = c[2 * (n_max - 1)];
    if (n_max <= 32) {
        for (int i = 1; i <= 31; ++i) {
            if (i < n_max) {
                out[2 * i] = c[2 * i];
                out[2 * i + 1] = c[2 * i + 1] / rate;
            } else {
                out[2 * i] = (double)(i + 1);
                out[2 * i + 1] = 1.0;
            }
        }
    } else if (n_max < 100) {
        for (int i = 1; i <= 7; ++i) {
            out[2 * i] = c[2 * i];
            out[2 * i + 1] = c[2 * i + 1] / rate;
        }
        double delta = (log((double)n_max) - log(9.0)) / (31.0 - 8.0);
        for (int i = 8; i <= 31; ++i) {
            double n = fmin(exp(log(9.0) + (double)(i - 8) * delta), limit);
            double v = 0.0;
            pw_evaluate(c, n_max, false, n, &v);
            out[2 * i] = n;
            out[2 * i + 1] = v / rate;
        }
    } else {
        double delta = log((double)n_max) / 31.0;
        for (int i = 1; i <= 31; ++i) {
            double n = fmin(exp((double)i * delta), limit);
            double v = 0.0;
            pw_evaluate(c, n_max, false, n, &v);
            out[2 * i] = n;
            out[2 * i + 1] = v / rate;
        }
    }
    total_out[p] = rate;
}

}  // namespace ptg

ptg_status ptg_regen_nlc_cp_cdf(ptg_ctx* c, double* cdf_out, double* total_out) {
    if (!c || !cdf_out || !total_out) return set_err(PTG_ERR_INVALID_ARGUMENT, "NULL argument");
    CUDA_TRY(cudaSetDevice(c->device));
    const int NC = 61, NR = 70, NP = NC * NR;
    std::vector<double> a_of(NP), eta_of(NP);
    std::vector<int> nmax_of(NP);
    std::vector<unsigned long long> off(NP);
    std::vector<RegenChunk> chunks;
    unsigned long long total_rows = 0;
    for (int i = 0; i < NR; ++i) {
        double eta = 1.0e-3 * std::pow(10.0, (double)i / 20.0);
        for (int j = 0; j < NC; ++j) {
            double a = 0.02 * std::pow(10.0, (double)j / 20.0);
            int p = i * NC + j;
            a_of[p] = a;
            eta_of[p] = eta;
            nmax_of[p] = (int)(10.0 * (1.0 + a * (a * a)));
            off[p] = total_rows;
            total_rows += nmax_of[p];
            for (int n0 = 1; n0 <= nmax_of[p]; n0 += 256) chunks.push_back(RegenChunk{p, n0});
        }
    }
    double *d_a = nullptr, *d_eta = nullptr, *d_rates = nullptr, *d_cum = nullptr, *d_cdf = nullptr, *d_tot = nullptr;
    int* d_nmax = nullptr;
    unsigned long long* d_off = nullptr;
    RegenChunk* d_chunks = nullptr;
    auto cleanup = [&]() {
        cudaFree(d_a), cudaFree(d_eta), cudaFree(d_rates), cudaFree(d_cum), cudaFree(d_cdf), cudaFree(d_tot);
        cudaFree(d_nmax), cudaFree(d_off), cudaFree(d_chunks);
    };
    bool ok = cudaMalloc(&d_a, 8 * NP) == cudaSuccess && cudaMalloc(&d_eta, 8 * NP) == cudaSuccess &&
              cudaMalloc(&d_nmax, 4 * NP) == cudaSuccess && cudaMalloc(&d_off, 8 * NP) == cudaSuccess &&
              cudaMalloc(&d_rates, 8 * total_rows) == cudaSuccess && cudaMalloc(&d_cum, 16 * total_rows) == cudaSuccess &&
              cudaMalloc(&d_cdf, 8 * 64 * NP) == cudaSuccess && cudaMalloc(&d_tot, 8 * NP) == cudaSuccess &&
              cudaMalloc(&d_chunks, sizeof(RegenChunk) * chunks.size()) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        cleanup();
        return set_err(PTG_ERR_ALLOC, "table regeneration buffers");
    }
    cudaMemcpy(d_a, a_of.data(), 8 * NP, cudaMemcpyHostToDevice);
    cudaMemcpy(d_eta, eta_of.data(), 8 * NP, cudaMemcpyHostToDevice);
    cudaMemcpy(d_nmax, nmax_of.data(), 4 * NP, cudaMemcpyHostToDevice);
    cudaMemcpy(d_off, off.data(), 8 * NP, cudaMemcpyHostToDevice);
    cudaMemcpy(d_chunks, chunks.data(), sizeof(RegenChunk) * chunks.size(), cudaMemcpyHostToDevice);
    k_regen_cp_partial<<<(unsigned)chunks.size(), 256, 0, c->stream>>>(d_chunks, d_a, d_eta, d_nmax, d_off, d_rates);
    k_regen_cp_cdf<<<(NP + 63) / 64, 64, 0, c->stream>>>(NP, d_nmax, d_off, d_rates, d_cum, d_cdf, d_tot);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) {
        cudaMemcpy(cdf_out, d_cdf, 8 * 64 * NP, cudaMemcpyDeviceToHost);
        cudaMemcpy(total_out, d_tot, 8 * NP, cudaMemcpyDeviceToHost);
    }
    cleanup();
    if (e != cudaSuccess) return set_err(PTG_ERR_CUDA, cudaGetErrorString(e));
    return PTG_OK;
}


ptg_status ptg_regen_bw_lp_mid_cdf(ptg_ctx* c, double* cdf_out, double* total_out) {
    if (!c || !cdf_out || !total_out) return set_err(PTG_ERR_INVALID_ARGUMENT, "NULL argument");
    CUDA_TRY(cudaSetDevice(c->device));
    const int NC = 36, NR = 157, NP = NC * NR;
    std::vector<int> nmin(NP), nmax(NP);
    std::vector<unsigned long long> off(NP);
    std::vector<int> n_of;
    std::vector<double> a_of, eta_of;
    int n_top = 1;
    for (int i = 0; i < NR; ++i) {
        double ep = std::exp(PTG_BW_LPM_LN_MAX_ETA_PRIME) / (1.0 + (double)i / PTG_BW_LPM_ETA_PRIME_DENSITY);
        for (int j = 0; j < NC; ++j) {
            double a = std::exp(PTG_BW_LPM_LN_MIN_A) * std::pow(10.0, (double)j / 20.0);
            double eta = (1.0 + 0.5 * a * a) * ep;
            int p = i * NC + j;
            lpp_sum_limits(a, eta, &nmin[p], &nmax[p]);
            if (nmax[p] < nmin[p]) nmax[p] = nmin[p];
            off[p] = n_of.size();
            for (int n = nmin[p]; n <= nmax[p]; ++n) {
                n_of.push_back(n);
                a_of.push_back(a);
                eta_of.push_back(eta);
                n_top = std::max(n_top, n);
            }
        }
    }
    size_t jobs = n_of.size();
    int cap = db_len_for(n_top);
    const size_t chunk = 32768;
    int *d_n = nullptr, *d_nmin = nullptr, *d_nmax = nullptr, *d_bad = nullptr;
    double *d_a = nullptr, *d_eta = nullptr, *d_rates = nullptr, *d_ws = nullptr, *d_cdf = nullptr, *d_tot = nullptr;
    unsigned long long* d_off = nullptr;
    auto cleanup = [&]() {
        cudaFree(d_n), cudaFree(d_nmin), cudaFree(d_nmax), cudaFree(d_bad), cudaFree(d_a), cudaFree(d_eta);
        cudaFree(d_rates), cudaFree(d_ws), cudaFree(d_cdf), cudaFree(d_tot), cudaFree(d_off);
    };
    bool ok = cudaMalloc(&d_n, 4 * jobs) == cudaSuccess && cudaMalloc(&d_a, 8 * jobs) == cudaSuccess &&
              cudaMalloc(&d_eta, 8 * jobs) == cudaSuccess && cudaMalloc(&d_rates, 16 * jobs) == cudaSuccess &&
              cudaMalloc(&d_ws, (size_t)cap * 40 * chunk) == cudaSuccess && cudaMalloc(&d_nmin, 4 * NP) == cudaSuccess &&
              cudaMalloc(&d_nmax, 4 * NP) == cudaSuccess && cudaMalloc(&d_off, 8 * NP) == cudaSuccess &&
              cudaMalloc(&d_cdf, 8 * 48 * NP) == cudaSuccess && cudaMalloc(&d_tot, 16 * NP) == cudaSuccess &&
              cudaMalloc(&d_bad, 4) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        cleanup();
        return set_err(PTG_ERR_ALLOC, "table regeneration buffers");
    }
    cudaMemcpy(d_n, n_of.data(), 4 * jobs, cudaMemcpyHostToDevice);
    cudaMemcpy(d_a, a_of.data(), 8 * jobs, cudaMemcpyHostToDevice);
    cudaMemcpy(d_eta, eta_of.data(), 8 * jobs, cudaMemcpyHostToDevice);
    cudaMemcpy(d_nmin, nmin.data(), 4 * NP, cudaMemcpyHostToDevice);
    cudaMemcpy(d_nmax, nmax.data(), 4 * NP, cudaMemcpyHostToDevice);
    cudaMemcpy(d_off, off.data(), 8 * NP, cudaMemcpyHostToDevice);
    cudaMemset(d_bad, 0, 4);
    cudaError_t e = cudaSuccess;
    for (size_t first = 0; first < jobs && e == cudaSuccess; first += chunk) {
        size_t count = std::min(chunk, jobs - first);
        e = launch_regen_lpm_partial(first, count, d_n, d_a, d_eta, d_ws, cap, d_rates, d_bad, c->stream);
    }
    if (e == cudaSuccess) e = launch_regen_lpm_cdf(NP, d_nmin, d_nmax, d_off, d_rates, d_cdf, d_tot, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    int bad = 0;
    if (e == cudaSuccess) {
        cudaMemcpy(&bad, d_bad, 4, cudaMemcpyDeviceToHost);
        cudaMemcpy(cdf_out, d_cdf, 8 * 48 * NP, cudaMemcpyDeviceToHost);
        cudaMemcpy(total_out, d_tot, 16 * NP, cudaMemcpyDeviceToHost);
    }
    cleanup();
    if (e != cudaSuccess) return set_err(PTG_ERR_CUDA, cudaGetErrorString(e));
    if (bad) return set_err(PTG_ERR_UNSUPPORTED, "harmonic beyond the J(n, x, y) workspace during regeneration");
    return PTG_OK;
}


// FP64 FMA throughput: eight independent chains per thread, so that the
// pipe, not the dependency latency, bounds it.
__global__ void k_fp64_fma(int iters, double a, double b, double* sink) {
    double x[8];
    for (int k = 0; k < 8; ++k) x[k] = 1.0 + 1e-3 * (threadIdx.x + k);
    for (int i = 0; i < iters; ++i)
        for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
    double acc = 0.0;
    for (int k = 0; k < 8; ++k) acc += x[k];
    if (acc == 12345.678) sink[0] = acc;  // keeps the chains live
}

// ------------------------------------------------- distribution output ---
// hgram.rs:171-184
static uint64_t hgram_number_of_bins(double mn, double mx, uint64_t n, const ptg_hgram_spec& sp) {
    if (mn == mx) return 1;
    switch (sp.bin_spec) {
        case PTG_BINS_FIXED_NUMBER: return (uint64_t)std::max(sp.n_bins, 0);
        case PTG_BINS_FIXED_SIZE: {
            double b = std::ceil((mx - mn) / sp.bin_size);
            return b > 0.0 ? (b < 1.8e19 ? (uint64_t)b : ~0ull) : 0;
        }
        default: {
            double b = std::ceil(2.0 * std::cbrt((double)n));
            return b > 0.0 ? (uint64_t)b : 0;
        }
    }
}

// the width of a bin along an axis (hgram.rs:186-205, 241-251)
static double hgram_bin_width(double mn, double mx, uint64_t nbins, const ptg_hgram_spec& sp) {
    return sp.bin_spec == PTG_BINS_FIXED_SIZE ? sp.bin_size : (mx - mn) / (double)nbins;
}

ptg_status ptg_histogram(ptg_ctx* c, const ptg_particles* d, const ptg_hgram_spec* sp, ptg_hgram_info* info,
                         double* counts, uint64_t counts_capacity) {
    if (!c || !d || !sp || !info) return set_err(PTG_ERR_INVALID_ARGUMENT, "NULL argument");
    if (sp->dim != 1 && sp->dim != 2) return set_err(PTG_ERR_INVALID_ARGUMENT, "histograms are 1- or 2-dimensional");
    for (int k = 0; k < sp->dim; ++k)
        if (sp->func[k] < PTG_OUT_ANGLE_X || sp->func[k] > PTG_OUT_HELICITY)
            return set_err(PTG_ERR_INVALID_ARGUMENT, "output function out of range");
    if (sp->filter_func < -1 || sp->filter_func > PTG_OUT_HELICITY || sp->weight < PTG_WEIGHT_NUMBER ||
        sp->weight > PTG_WEIGHT_HELICITY || sp->bin_spec < PTG_BINS_AUTO || sp->bin_spec > PTG_BINS_FIXED_SIZE ||
        sp->height < PTG_HEIGHT_COUNT || sp->height > PTG_HEIGHT_PDF)
        return set_err(PTG_ERR_INVALID_ARGUMENT, "histogram specification out of range");
    if (sp->bin_spec == PTG_BINS_FIXED_NUMBER && sp->n_bins < 1)
        return set_err(PTG_ERR_INVALID_ARGUMENT, "a fixed number of bins must be >= 1");
    if (sp->bin_spec == PTG_BINS_FIXED_SIZE && !(sp->bin_size > 0.0))
        return set_err(PTG_ERR_INVALID_ARGUMENT, "a fixed bin size must be > 0");
    if (d->n == 0) {
        // no particles: an empty histogram (the reference writes none)
        std::memset(info, 0, sizeof(*info));
        info->dim = sp->dim;
        info->empty = 1;
        return PTG_OK;
    }
    if (!d->species || !d->u || !d->r || !d->pol || !d->weight)
        return set_err(PTG_ERR_INVALID_ARGUMENT, "particles need species, u, r, pol and weight");
    auto uses = [&](int f) {
        if (sp->filter_func == f) return true;
        for (int k = 0; k < sp->dim; ++k)
            if (sp->func[k] == f) return true;
        return false;
    };
    if ((uses(PTG_OUT_PAYLOAD) && !d->payload) || (uses(PTG_OUT_PARENT_CHI) && !d->parent_chi) ||
        (uses(PTG_OUT_N_INTER) && !d->interaction_count) || (uses(PTG_OUT_ABSORPTION) && !d->work))
        return set_err(PTG_ERR_INVALID_ARGUMENT, "an output function reads a field that is NULL");
    std::memset(info, 0, sizeof(*info));
    info->dim = sp->dim;
    CUDA_TRY(cudaSetDevice(c->device));
    HgramArgs h{};
    h.species = d->species, h.u = d->u, h.r = d->r, h.pol = d->pol, h.weight = d->weight;
    h.payload = d->payload, h.parent_chi = d->parent_chi, h.icount = d->interaction_count, h.work = d->work;
    h.n = d->n;
    h.want_species = sp->species;
    h.dim = sp->dim;
    h.func[0] = sp->func[0], h.func[1] = sp->dim == 2 ? sp->func[1] : sp->func[0];
    h.scale[0] = sp->scale[0], h.scale[1] = sp->dim == 2 ? sp->scale[1] : sp->scale[0];
    h.wfunc = sp->weight;
    h.log_bins = sp->bin_spec == PTG_BINS_LOG;
    h.filter_func = sp->filter_func;
    h.fmin = sp->filter_min, h.fmax = sp->filter_max;
    int blocks = (int)std::min<unsigned long long>((d->n + 255) / 256, 4ull * (unsigned long long)c->num_sms);
    if (blocks < 1) blocks = 1;
    double* dpart = nullptr;
    double* dcts = nullptr;
    auto cleanup = [&]() { cudaFree(dpart), cudaFree(dcts); };
    if (cudaMalloc(&dpart, 48 * (size_t)blocks) != cudaSuccess) {
        cudaGetLastError();
        return set_err(PTG_ERR_ALLOC, "histogram partials");
    }
    std::vector<double> part(6 * (size_t)blocks);
    cudaError_t e = launch_hgram_stats(h, blocks, dpart, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(part.data(), dpart, 48 * (size_t)blocks, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        cleanup();
        return set_err(PTG_ERR_CUDA, cudaGetErrorString(e));
    }
    double mn[2] = {DBL_MAX, DBL_MAX}, mx[2] = {-DBL_MAX, -DBL_MAX}, total = 0.0, num = 0.0;
    for (int b = 0; b < blocks; ++b) {
        const double* p = &part[6 * (size_t)b];
        mn[0] = std::min(mn[0], p[0]), mx[0] = std::max(mx[0], p[1]);
        mn[1] = std::min(mn[1], p[2]), mx[1] = std::max(mx[1], p[3]);
        total += p[4], num += p[5];
    }
    uint64_t gnum = (uint64_t)num;
    if (gnum == 0) {
        info->empty = 1;
        cleanup();
        return PTG_OK;
    }
    // bins, sizes and the bin volume (hgram.rs:240-251 in 1d, 186-205 in 2d)
    double vol = 1.0;
    for (int k = 0; k < sp->dim; ++k) {
        uint64_t nb = hgram_number_of_bins(mn[k], mx[k], gnum, *sp);
        info->bins[k] = nb;
        info->min[k] = mn[k], info->max[k] = mx[k];
        double w = mn[k] == mx[k] ? (sp->dim == 1 ? 1.0 : 0.0) : hgram_bin_width(mn[k], mx[k], nb, *sp);
        if (sp->dim == 1) {
            vol = w;
            h.bin_sz[0] = w;
            info->bin_size[0] = nb <= 1 ? 0.0 : w;
        } else {
            vol *= mn[k] == mx[k] ? 1.0 : w;
            h.bin_sz[k] = w;
            info->bin_size[k] = w;
        }
        h.gmin[k] = mn[k];
        h.nbins[k] = nb;
    }
    if (sp->dim == 1) info->bins[1] = 1, h.nbins[1] = 1;
    unsigned long long ncts = h.nbins[0] * h.nbins[1];
    if (h.nbins[0] == 0 || h.nbins[1] == 0 || h.nbins[0] > (1ull << 31) || h.nbins[1] > (1ull << 31) ||
        ncts > (1ull << 31)) {
        cleanup();
        return set_err(PTG_ERR_INVALID_ARGUMENT, "histogram would have " + std::to_string(h.nbins[0]) + " x " +
                                                     std::to_string(h.nbins[1]) + " bins");
    }
    info->n_counts = ncts;
    info->bin_volume = vol;
    info->total = total;
    info->unweighted_total = (double)gnum;
    if (!counts || counts_capacity < ncts) {
        cleanup();
        return PTG_OK;
    }
    h.density_log = h.log_bins && (sp->height == PTG_HEIGHT_DENSITY || sp->height == PTG_HEIGHT_PDF);
    if (cudaMalloc(&dcts, 8 * ncts) != cudaSuccess) {
        cudaGetLastError();
        cleanup();
        return set_err(PTG_ERR_ALLOC, "histogram counts");
    }
    e = cudaMemsetAsync(dcts, 0, 8 * ncts, c->stream);
    if (e == cudaSuccess) e = launch_hgram_fill(h, blocks, dcts, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(counts, dcts, 8 * ncts, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cleanup();
    if (e != cudaSuccess) return set_err(PTG_ERR_CUDA, cudaGetErrorString(e));
    // heights (hgram.rs:297-301)
    if (sp->height == PTG_HEIGHT_DENSITY)
        for (unsigned long long k = 0; k < ncts; ++k) counts[k] = counts[k] / vol;
    else if (sp->height == PTG_HEIGHT_PDF)
        for (unsigned long long k = 0; k < ncts; ++k) counts[k] = counts[k] / (vol * total);
    return PTG_OK;
}

ptg_status ptg_particle_sums(ptg_ctx* c, const ptg_particles* d, const ptg_stats_spec* sp, ptg_stats_sums* out) {
    if (!c || !d || !sp || !out) return set_err(PTG_ERR_INVALID_ARGUMENT, "NULL argument");
    for (int f : {sp->var_func, sp->weight_func})
        if (f < PTG_OUT_ANGLE_X || f > PTG_OUT_HELICITY)
            return set_err(PTG_ERR_INVALID_ARGUMENT, "output function out of range");
    if (sp->filter_func < -1 || sp->filter_func > PTG_OUT_HELICITY)
        return set_err(PTG_ERR_INVALID_ARGUMENT, "filter function out of range");
    if (d->n == 0) {
        // no particles: the sums of an empty set
        *out = ptg_stats_sums{0.0, 0.0, 0.0, HUGE_VAL, -HUGE_VAL, 0.0, 0.0, 0.0, 0.0};
        return PTG_OK;
    }
    if (!d->species || !d->u || !d->r || !d->pol || !d->weight)
        return set_err(PTG_ERR_INVALID_ARGUMENT, "particles need species, u, r, pol and weight");
    for (int f : {sp->var_func, sp->weight_func, sp->filter_func})
        if ((f == PTG_OUT_PAYLOAD && !d->payload) || (f == PTG_OUT_PARENT_CHI && !d->parent_chi) ||
            (f == PTG_OUT_N_INTER && !d->interaction_count) || (f == PTG_OUT_ABSORPTION && !d->work))
            return set_err(PTG_ERR_INVALID_ARGUMENT, "an output function reads a field that is NULL");
    CUDA_TRY(cudaSetDevice(c->device));
    HgramArgs h{};
    h.species = d->species, h.u = d->u, h.r = d->r, h.pol = d->pol, h.weight = d->weight;
    h.payload = d->payload, h.parent_chi = d->parent_chi, h.icount = d->interaction_count, h.work = d->work;
    h.n = d->n;
    h.want_species = sp->species;
    h.func[0] = sp->var_func, h.func[1] = sp->weight_func;
    h.filter_func = sp->filter_func;
    h.fmin = sp->min, h.fmax = sp->max;
    int blocks = (int)std::min<unsigned long long>((d->n + 255) / 256, 4ull * (unsigned long long)c->num_sms);
    if (blocks < 1) blocks = 1;
    double* dpart = nullptr;
    if (cudaMalloc(&dpart, 72 * (size_t)blocks) != cudaSuccess) {
        cudaGetLastError();
        return set_err(PTG_ERR_ALLOC, "statistic partials");
    }
    std::vector<double> part(9 * (size_t)blocks);
    cudaError_t e = launch_particle_sums(h, sp->shift, blocks, dpart, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(part.data(), dpart, 72 * (size_t)blocks, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(dpart);
    if (e != cudaSuccess) return set_err(PTG_ERR_CUDA, cudaGetErrorString(e));
    double a[9] = {0.0, 0.0, 0.0, HUGE_VAL, -HUGE_VAL, 0.0, 0.0, 0.0, 0.0};
    for (int b = 0; b < blocks; ++b)
        for (int k = 0; k < 9; ++k) {
            double v = part[9 * (size_t)b + k];
            a[k] = k == 3 ? std::min(a[k], v) : (k == 4 ? std::max(a[k], v) : a[k] + v);
        }
    out->total = a[0], out->subtotal = a[1], out->count = a[2], out->minimum = a[3], out->maximum = a[4];
    out->sum_diffs = a[5], out->sum_sq_diffs = a[6], out->sum_cos = a[7], out->sum_sin = a[8];
    return PTG_OK;
}

// ------------------------------------------------------ beam builder ---
ptg_status ptg_build_beam(ptg_ctx* c, const ptg_beam_desc* d, uint64_t n, uint64_t seed, uint64_t first_id,
                          const ptg_particles* out) {
    if (!c || !d || !out) return set_err(PTG_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n == 0) return PTG_OK;
    if (d->species < PTG_ELECTRON || d->species > PTG_PHOTON)
        return set_err(PTG_ERR_INVALID_ARGUMENT, "beam species out of range");
    if (d->gamma_dstr < PTG_GAMMA_NORMAL || d->gamma_dstr > PTG_GAMMA_CUSTOM || d->radial_dstr < PTG_RADIAL_NORMAL ||
        d->radial_dstr > PTG_RADIAL_UNIFORM)
        return set_err(PTG_ERR_INVALID_ARGUMENT, "beam distribution out of range");
    if (!(std::fabs(d->energy_chirp) < 1.0)) return set_err(PTG_ERR_INVALID_ARGUMENT, "energy chirp must lie in (-1, 1)");
    if (d->gamma_dstr == PTG_GAMMA_NORMAL && !(d->gamma_mean > 1.0 && d->gamma_sigma >= 0.0))
        return set_err(PTG_ERR_INVALID_ARGUMENT, "normal spectrum needs gamma > 1 and sigma >= 0");
    if (d->gamma_dstr == PTG_GAMMA_BREM && !(d->gamma_min > 0.0 && d->gamma_max > d->gamma_min))
        return set_err(PTG_ERR_INVALID_ARGUMENT, "bremsstrahlung spectrum needs 0 < gamma_min < gamma_max");
    if (d->gamma_dstr == PTG_GAMMA_CUSTOM) {
        if (!d->custom_cdf || d->custom_len < 2 || d->custom_len > 4096)
            return set_err(PTG_ERR_INVALID_ARGUMENT, "custom spectrum needs 2..4096 CDF nodes");
        for (int k = 0; k < d->custom_len; ++k) {
            const double* p = d->custom_cdf + 2 * k;
            if (!std::isfinite(p[0]) || !std::isfinite(p[1]) ||
                (k > 0 && (p[0] <= p[-2] || p[1] < p[-1])))
                return set_err(PTG_ERR_INVALID_ARGUMENT, "custom CDF nodes must be finite and increasing");
        }
    }
    if (d->radial_dstr == PTG_RADIAL_TRUNC_NORMAL && !(d->x_max > 0.0 && d->y_max > 0.0))
        return set_err(PTG_ERR_INVALID_ARGUMENT, "truncated normal needs x_max, y_max > 0");
    CUDA_TRY(cudaSetDevice(c->device));
    BeamArgs b{};
    b.species = d->species;
    b.gamma_dstr = d->gamma_dstr;
    b.radial_dstr = d->radial_dstr;
    b.gamma_mean = d->gamma_mean, b.gamma_sigma = d->gamma_sigma;
    b.gamma_min = d->gamma_min, b.gamma_max = d->gamma_max;
    b.rho = -d->energy_chirp;  // builder.rs:120-124 flips the sign
    b.sigma_x = d->sigma_x, b.sigma_y = d->sigma_y, b.x_max = d->x_max, b.y_max = d->y_max, b.r_max = d->r_max;
    b.sigma_z = d->sigma_z, b.rms_div = d->rms_div;
    b.angle = d->collision_angle;
    b.cos_a = std::cos(d->collision_angle), b.sin_a = std::sin(d->collision_angle);
    b.cos_p = std::cos(d->collision_plane), b.sin_p = std::sin(d->collision_plane);
    b.off_x = d->offset[0], b.off_y = d->offset[1], b.off_z = d->offset[2];
    b.initial_z = d->initial_z;
    for (int k = 0; k < 4; ++k) b.pol[k] = d->pol[k];
    b.weight = d->weight;
    double* dcdf = nullptr;
    unsigned long long* derr = nullptr;
    auto cleanup = [&]() { cudaFree(dcdf), cudaFree(derr); };
    if (cudaMalloc(&derr, 8) != cudaSuccess) {
        cudaGetLastError();
        return set_err(PTG_ERR_ALLOC, "beam builder counter");
    }
    if (d->gamma_dstr == PTG_GAMMA_CUSTOM) {
        if (cudaMalloc(&dcdf, 16 * (size_t)d->custom_len) != cudaSuccess) {
            cudaGetLastError();
            cleanup();
            return set_err(PTG_ERR_ALLOC, "custom spectrum table");
        }
        cudaMemcpyAsync(dcdf, d->custom_cdf, 16 * (size_t)d->custom_len, cudaMemcpyHostToDevice, c->stream);
        b.custom_cdf = dcdf;
        b.custom_len = d->custom_len;
    }
    cudaMemsetAsync(derr, 0, 8, c->stream);
    cudaError_t e = launch_build_beam(b, n, seed, first_id, out->species, out->r, out->u, out->pol, out->weight,
                                      (unsigned long long*)out->id, (unsigned long long*)out->parent_id, derr,
                                      c->stream);
    unsigned long long nerr = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&nerr, derr, 8, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cleanup();
    if (e != cudaSuccess) return set_err(PTG_ERR_CUDA, cudaGetErrorString(e));
    if (nerr) return set_err(PTG_ERR_REJECTION_CAP, std::to_string(nerr) + " primaries could not be sampled");
    return PTG_OK;
}

// One FP64 library function per kernel, called `iters` times by every
// thread on inputs inside all the functions' domains, so that a profiler's
// FP64 instruction counts per launch, less those of PTG_FN_NONE, divided by
// the calls, give each function's executed cost on this device.
template <int OP>
__device__ __forceinline__ double fp64_fn(double x) {
    switch (OP) {
        case PTG_FN_EXP: return exp(-x);
        case PTG_FN_LOG: return log(x);
        case PTG_FN_DIV: return 1.0 / x;
        case PTG_FN_SQRT: return sqrt(x);
        case PTG_FN_CBRT: return cbrt(x);
        case PTG_FN_SINCOS: {
            double s, c;
            sincos(x, &s, &c);
            return s + c;
        }
        case PTG_FN_POW: return pow(x, 1.0 / 6.0);
        case PTG_FN_ATAN2: return atan2(x, 1.3);
        case PTG_FN_HYPOT: return hypot(x, 1.3);
        case PTG_FN_LOG1P: return log1p(x);
        case PTG_FN_ACOS: return acos(x);
        default: return x;
    }
}

template <int OP>
__global__ void k_fp64_fn(int iters, double x0, double* sink) {
    double x = x0 + 1e-9 * (double)(blockIdx.x * blockDim.x + threadIdx.x);
    double acc = 0.0;
    for (int i = 0; i < iters; ++i) {
        acc += fp64_fn<OP>(x);
        x += 1e-12;
    }
    if (acc == 12345.678) *sink = acc;  // keeps the loop; never true
}

ptg_status ptg_fp64_function_kernel(ptg_ctx* c, int32_t op, int32_t iters) {
    if (!c) return set_err(PTG_ERR_INVALID_ARGUMENT, "ctx is NULL");
    if (iters < 1 || iters > (1 << 20)) return set_err(PTG_ERR_INVALID_ARGUMENT, "iters out of range");
    CUDA_TRY(cudaSetDevice(c->device));
    double* sink = nullptr;
    CUDA_TRY(cudaMalloc(&sink, 8));
    const int block = 256, grid = c->num_sms;
    const double x0 = 0.37;
    switch (op) {
        case PTG_FN_NONE: k_fp64_fn<PTG_FN_NONE><<<grid, block, 0, c->stream>>>(iters, x0, sink); break;
        case PTG_FN_EXP: k_fp64_fn<PTG_FN_EXP><<<grid, block, 0, c->stream>>>(iters, x0, sink); break;
        case PTG_FN_LOG: k_fp64_fn<PTG_FN_LOG><<<grid, block, 0, c->stream>>>(iters, x0, sink); break;
        case PTG_FN_DIV: k_fp64_fn<PTG_FN_DIV><<<grid, block, 0, c->stream>>>(iters, x0, sink); break;
        case PTG_FN_SQRT: k_fp64_fn<PTG_FN_SQRT><<<grid, block, 0, c->stream>>>(iters, x0, sink); break;
        case PTG_FN_CBRT: k_fp64_fn<PTG_FN_CBRT><<<grid, block, 0, c->stream>>>(iters, x0, sink); break;
        case PTG_FN_SINCOS: k_fp64_fn<PTG_FN_SINCOS><<<grid, block, 0, c->stream>>>(iters, x0, sink); break;
        case PTG_FN_POW: k_fp64_fn<PTG_FN_POW><<<grid, block, 0, c->stream>>>(iters, x0, sink); break;
        case PTG_FN_ATAN2: k_fp64_fn<PTG_FN_ATAN2><<<grid, block, 0, c->stream>>>(iters, x0, sink); break;
        case PTG_FN_HYPOT: k_fp64_fn<PTG_FN_HYPOT><<<grid, block, 0, c->stream>>>(iters, x0, sink); break;
        case PTG_FN_LOG1P: k_fp64_fn<PTG_FN_LOG1P><<<grid, block, 0, c->stream>>>(iters, x0, sink); break;
        case PTG_FN_ACOS: k_fp64_fn<PTG_FN_ACOS><<<grid, block, 0, c->stream>>>(iters, x0, sink); break;
        default:
            cudaFree(sink);
            return set_err(PTG_ERR_INVALID_ARGUMENT, "unknown function");
    }
    cudaError_t e = cudaStreamSynchronize(c->stream);
    cudaFree(sink);
    if (e != cudaSuccess) return set_err(PTG_ERR_CUDA, cudaGetErrorString(e));
    return PTG_OK;
}

ptg_status ptg_fp64_peak(ptg_ctx* c, double* tflops) {
    if (!c || !tflops) return set_err(PTG_ERR_INVALID_ARGUMENT, "NULL argument");
    CUDA_TRY(cudaSetDevice(c->device));
    double* sink = nullptr;
    CUDA_TRY(cudaMalloc(&sink, 8));
    const int iters = 4096, block = 256, grid = 8 * c->num_sms;
    k_fp64_fma<<<grid, block, 0, c->stream>>>(iters, 0.999999, 1e-9, sink);
    CUDA_TRY(cudaEventRecord(c->ev0, c->stream));
    for (int r = 0; r < 5; ++r) k_fp64_fma<<<grid, block, 0, c->stream>>>(iters, 0.999999, 1e-9, sink);
    CUDA_TRY(cudaEventRecord(c->ev1, c->stream));
    CUDA_TRY(cudaEventSynchronize(c->ev1));
    float ms = 0.0f;
    CUDA_TRY(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    cudaFree(sink);
    *tflops = 5.0 * 2.0 * 8.0 * iters * (double)grid * block / (ms * 1e-3) / 1e12;
    return PTG_OK;
}


// ---------------------------------------------------- learned proposal ---
static const int MLP_GRAD_BLOCKS = 304;  // two per SM on 152 SMs (shared memory allows two)

static MlpDev mlp_dev(ptg_ctx* c) {
    MlpDev m{};
    __nv_bfloat16* b = c->mlp_bf;
    m.w0 = b;
    m.w1 = m.w0 + MLP_H * MLP_IN_PAD;
    m.w2 = m.w1 + MLP_H * MLP_H;
    m.w3 = m.w2 + MLP_H * MLP_H;
    m.t1 = m.w3 + MLP_OUT * MLP_H;
    m.t2 = m.t1 + MLP_H * MLP_H;
    m.t3 = m.t2 + MLP_H * MLP_H;
    m.p = c->mlp_p;
    return m;
}

// The collision kernels' view (disabled unless a trained network is in use).
static MlpParams mlp_params(ptg_ctx* c) {
    MlpParams p{};
    if (!c->mlp_ready || !c->mlp_enabled) return p;
    MlpDev m = mlp_dev(c);
    p.w0 = m.w0, p.w1 = m.w1, p.w2 = m.w2, p.w3 = m.w3;
    p.b0 = c->mlp_p + P_B0, p.b1 = c->mlp_p + P_B1, p.b2 = c->mlp_p + P_B2, p.b3 = c->mlp_p + P_B3;
    p.margin = c->mlp_margin;
    p.enabled = 1;
    p.min_harmonic = c->mlp_min_harmonic;
    return p;
}

static ptg_status mlp_alloc(ptg_ctx* c) {
    if (c->mlp_p) return PTG_OK;
    size_t np = P_TOTAL;
    // w0, w1, w2, w3 and the transposes t1, t2, t3 (mlp_dev's layout)
    size_t nbf = (size_t)MLP_H * MLP_IN_PAD + 4 * (size_t)MLP_H * MLP_H + 2 * (size_t)MLP_OUT * MLP_H;
    if (cudaMalloc(&c->mlp_p, 4 * np) != cudaSuccess || cudaMalloc(&c->mlp_m, 4 * np) != cudaSuccess ||
        cudaMalloc(&c->mlp_v, 4 * np) != cudaSuccess ||
        cudaMalloc(&c->mlp_partial, 4 * np * MLP_GRAD_BLOCKS) != cudaSuccess ||
        cudaMalloc(&c->mlp_loss, 4 * MLP_GRAD_BLOCKS) != cudaSuccess || cudaMalloc(&c->mlp_bf, 2 * nbf) != cudaSuccess ||
        cudaMalloc(&c->mlp_packed, mlp_packed_bytes()) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(c->mlp_p), cudaFree(c->mlp_m), cudaFree(c->mlp_v), cudaFree(c->mlp_partial), cudaFree(c->mlp_loss);
        cudaFree(c->mlp_bf), cudaFree(c->mlp_packed);
        c->mlp_p = c->mlp_m = c->mlp_v = c->mlp_partial = c->mlp_loss = nullptr;
        c->mlp_bf = nullptr;
        c->mlp_packed = nullptr;
        return set_err(PTG_ERR_ALLOC, "learned-proposal buffers");
    }
    CUDA_TRY(cudaMemset(c->mlp_bf, 0, 2 * nbf));
    return PTG_OK;
}

ptg_status ptg_mlp_init(ptg_ctx* c, uint64_t seed) {
    if (!c) return set_err(PTG_ERR_INVALID_ARGUMENT, "ctx is NULL");
    CUDA_TRY(cudaSetDevice(c->device));
    ptg_status st = mlp_alloc(c);
    if (st != PTG_OK) return st;
    // uniform He initialisation from a splitmix sequence; biases zero
    std::vector<float> p(P_TOTAL, 0.0f);
    uint64_t z = seed;
    auto uni = [&]() {
        z += 0x9E3779B97F4A7C15ull;
        uint64_t x = z;
        x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
        x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
        x ^= x >> 31;
        return (double)(x >> 11) * (1.0 / 9007199254740992.0);
    };
    auto fill = [&](int off, int rows, int cols, int used_cols, int fan_in) {
        double lim = std::sqrt(6.0 / fan_in);
        for (int r = 0; r < rows; ++r)
            for (int k = 0; k < cols; ++k)
                p[off + r * cols + k] = k < used_cols ? (float)((2.0 * uni() - 1.0) * lim) : 0.0f;
    };
    fill(P_W0, MLP_H, MLP_IN_PAD, MLP_IN, MLP_IN);
    fill(P_W1, MLP_H, MLP_H, MLP_H, MLP_H);
    fill(P_W2, MLP_H, MLP_H, MLP_H, MLP_H);
    fill(P_W3, MLP_OUT, MLP_H, MLP_H, MLP_H);
    CUDA_TRY(cudaMemcpy(c->mlp_p, p.data(), 4 * P_TOTAL, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemset(c->mlp_m, 0, 4 * P_TOTAL));
    CUDA_TRY(cudaMemset(c->mlp_v, 0, 4 * P_TOTAL));
    c->mlp_step = 0;
    CUDA_TRY(launch_mlp_sync(c->mlp_p, mlp_dev(c), c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->mlp_ready = true;
    return PTG_OK;
}

ptg_status ptg_mlp_params(ptg_ctx* c, float* get, const float* set, int32_t* count) {
    if (!c) return set_err(PTG_ERR_INVALID_ARGUMENT, "ctx is NULL");
    if (count) *count = P_TOTAL;
    if (!get && !set) return PTG_OK;
    CUDA_TRY(cudaSetDevice(c->device));
    ptg_status st = mlp_alloc(c);
    if (st != PTG_OK) return st;
    if (set) {
        std::vector<float> p(set, set + P_TOTAL);
        for (int r = 0; r < MLP_H; ++r)
            for (int k = MLP_IN; k < MLP_IN_PAD; ++k) p[P_W0 + r * MLP_IN_PAD + k] = 0.0f;
        CUDA_TRY(cudaMemcpy(c->mlp_p, p.data(), 4 * P_TOTAL, cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemset(c->mlp_m, 0, 4 * P_TOTAL));
        CUDA_TRY(cudaMemset(c->mlp_v, 0, 4 * P_TOTAL));
        c->mlp_step = 0;
        CUDA_TRY(launch_mlp_sync(c->mlp_p, mlp_dev(c), c->stream));
        CUDA_TRY(cudaStreamSynchronize(c->stream));
        c->mlp_ready = true;
    }
    if (get) {
        if (!c->mlp_ready) return set_err(PTG_ERR_INVALID_ARGUMENT, "no network: call ptg_mlp_init or set parameters");
        CUDA_TRY(cudaMemcpy(get, c->mlp_p, 4 * P_TOTAL, cudaMemcpyDeviceToHost));
    }
    return PTG_OK;
}

ptg_status ptg_mlp_grad(ptg_ctx* c, const float* samples, size_t n, float tau, float* grad, float* loss) {
    if (!c || !samples || !grad) return set_err(PTG_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!c->mlp_ready) return set_err(PTG_ERR_INVALID_ARGUMENT, "no network: call ptg_mlp_init first");
    if (n == 0 || n > (1u << 24)) return set_err(PTG_ERR_INVALID_ARGUMENT, "sample count out of range");
    CUDA_TRY(cudaSetDevice(c->device));
    // rows of MLP_IN inputs, the bin (as a float) and the target
    const size_t row = MLP_IN + 2, sb = mlp_sample_bytes();
    std::vector<char> buf(sb * n);
    for (size_t i = 0; i < n; ++i) {
        const float* r = samples + row * i;
        int bin = (int)r[MLP_IN];
        std::memcpy(&buf[i * sb], r, 4 * MLP_IN);
        std::memcpy(&buf[i * sb + 4 * MLP_IN], &bin, 4);
        std::memcpy(&buf[i * sb + 4 * MLP_IN + 4], &r[MLP_IN + 1], 4);
    }
    void* d = nullptr;
    CUDA_TRY(cudaMalloc(&d, buf.size()));
    cudaMemcpy(d, buf.data(), buf.size(), cudaMemcpyHostToDevice);
    cudaError_t e = launch_mlp_grad(mlp_dev(c), d, 0, (int)n, tau, c->mlp_partial, c->mlp_loss, MLP_GRAD_BLOCKS, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    std::vector<float> part((size_t)P_TOTAL * MLP_GRAD_BLOCKS), ls(MLP_GRAD_BLOCKS);
    if (e == cudaSuccess) {
        cudaMemcpy(part.data(), c->mlp_partial, 4 * part.size(), cudaMemcpyDeviceToHost);
        cudaMemcpy(ls.data(), c->mlp_loss, 4 * ls.size(), cudaMemcpyDeviceToHost);
    }
    cudaFree(d);
    if (e != cudaSuccess) return set_err(PTG_ERR_CUDA, cudaGetErrorString(e));
    for (int i = 0; i < P_TOTAL; ++i) {
        double g = 0.0;
        for (int b = 0; b < MLP_GRAD_BLOCKS; ++b) g += part[(size_t)b * P_TOTAL + i];
        grad[i] = (float)g;
    }
    if (loss) {
        double l = 0.0;
        for (float v : ls) l += v;
        *loss = (float)(l / (double)n);
    }
    return PTG_OK;
}

ptg_status ptg_mlp_infer(ptg_ctx* c, const float* x, size_t n, float* out) {
    if (!c || !x || !out) return set_err(PTG_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!c->mlp_ready) return set_err(PTG_ERR_INVALID_ARGUMENT, "no network: call ptg_mlp_init first");
    if (n == 0) return PTG_OK;
    CUDA_TRY(cudaSetDevice(c->device));
    float *dx = nullptr, *dout = nullptr;
    CUDA_TRY(cudaMalloc(&dx, 4 * MLP_IN * n));
    if (cudaMalloc(&dout, 64 * n) != cudaSuccess) {
        cudaFree(dx);
        return set_err(PTG_ERR_ALLOC, "inference buffers");
    }
    cudaMemcpy(dx, x, 4 * MLP_IN * n, cudaMemcpyHostToDevice);
    cudaError_t e = launch_mlp_infer(mlp_dev(c), c->mlp_packed, dx, n, dout, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess) cudaMemcpy(out, dout, 64 * n, cudaMemcpyDeviceToHost);
    cudaFree(dx), cudaFree(dout);
    if (e != cudaSuccess) return set_err(PTG_ERR_CUDA, cudaGetErrorString(e));
    return PTG_OK;
}

ptg_status ptg_mlp_train(ptg_ctx* c, const ptg_mlp_train_cfg* cfg, ptg_mlp_train_stats* stats) {
    if (!c || !cfg) return set_err(PTG_ERR_INVALID_ARGUMENT, "NULL argument");
    if (cfg->n_samples < 1024 || cfg->batch < 64 || cfg->epochs < 1 || !(cfg->lr > 0.0f) ||
        !(cfg->tau > 0.0f && cfg->tau < 1.0f))
        return set_err(PTG_ERR_INVALID_ARGUMENT, "training configuration out of range");
    CUDA_TRY(cudaSetDevice(c->device));
    if (!c->tables_loaded) {
        ptg_status st = ptg_load_tables(c, nullptr);
        if (st != PTG_OK) return st;
    }
    if (!c->lma_host.nlc_cp_cdf) return set_err(PTG_ERR_TABLES, "the CP harmonic CDF table is needed");
    if (!c->mlp_ready) {
        ptg_status st = ptg_mlp_init(c, cfg->seed ^ 0x5DEECE66Dull);
        if (st != PTG_OK) return st;
    }
    void* data = nullptr;
    size_t bytes = mlp_sample_bytes() * cfg->n_samples;
    if (cudaMalloc(&data, bytes) != cudaSuccess) {
        cudaGetLastError();
        return set_err(PTG_ERR_ALLOC, "training data (" + std::to_string(bytes) + " bytes)");
    }
    CUDA_TRY(cudaEventRecord(c->ev0, c->stream));
    cudaError_t e = launch_mlp_data(c->lma_dev, cfg->n_samples, cfg->seed, cfg->a_lo, cfg->a_hi, cfg->eta_lo,
                                    cfg->eta_hi, data, c->stream);
    cudaEvent_t ev_mid = nullptr;
    cudaEventCreate(&ev_mid);
    cudaEventRecord(ev_mid, c->stream);
    unsigned long long steps_per_epoch = cfg->n_samples / (unsigned long long)cfg->batch;
    long long total = (long long)steps_per_epoch * cfg->epochs;
    float loss_first = NAN, loss_last = NAN;
    std::vector<float> ls(MLP_GRAD_BLOCKS);
    for (long long k = 0; k < total && e == cudaSuccess; ++k) {
        unsigned long long first = (unsigned long long)(k % (long long)steps_per_epoch) * cfg->batch;
        // cosine decay of the learning rate
        float lr = cfg->lr * 0.5f * (1.0f + std::cos(3.14159265f * (float)k / (float)total));
        e = launch_mlp_grad(mlp_dev(c), data, first, cfg->batch, cfg->tau, c->mlp_partial, c->mlp_loss,
                            MLP_GRAD_BLOCKS, c->stream);
        if (e == cudaSuccess)
            e = launch_mlp_adam(c->mlp_p, c->mlp_m, c->mlp_v, c->mlp_partial, MLP_GRAD_BLOCKS, lr, ++c->mlp_step,
                                mlp_dev(c), c->stream);
        if (e == cudaSuccess && (k == 0 || k == total - 1)) {
            e = cudaMemcpyAsync(ls.data(), c->mlp_loss, 4 * MLP_GRAD_BLOCKS, cudaMemcpyDeviceToHost, c->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
            double l = 0.0;
            for (float v : ls) l += v;
            (k == 0 ? loss_first : loss_last) = (float)(l / cfg->batch);
        }
    }
    cudaEventRecord(c->ev1, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    float ms_data = 0.0f, ms_all = 0.0f;
    cudaEventElapsedTime(&ms_data, c->ev0, ev_mid);
    cudaEventElapsedTime(&ms_all, c->ev0, c->ev1);
    cudaEventDestroy(ev_mid);
    cudaFree(data);
    if (e != cudaSuccess) return set_err(PTG_ERR_CUDA, cudaGetErrorString(e));
    if (stats) {
        stats->loss_first = loss_first;
        stats->loss_last = loss_last;
        stats->steps = (int32_t)total;
        stats->data_ms = ms_data;
        stats->train_ms = ms_all - ms_data;
    }
    return PTG_OK;
}

ptg_status ptg_mlp_use(ptg_ctx* c, int32_t enabled, float margin) {
    if (!c) return set_err(PTG_ERR_INVALID_ARGUMENT, "ctx is NULL");
    if (enabled && !c->mlp_ready) return set_err(PTG_ERR_INVALID_ARGUMENT, "no network: train or load one first");
    if (!(margin >= 0.0f && margin < 10.0f)) return set_err(PTG_ERR_INVALID_ARGUMENT, "margin out of range");
    c->mlp_enabled = enabled != 0;
    c->mlp_margin = margin;
    return PTG_OK;
}

ptg_status ptg_mlp_min_harmonic(ptg_ctx* c, int32_t n, int32_t* previous) {
    if (!c) return set_err(PTG_ERR_INVALID_ARGUMENT, "ctx is NULL");
    if (previous) *previous = c->mlp_min_harmonic;
    if (n < 0) return PTG_OK;  // query only
    c->mlp_min_harmonic = n;
    return PTG_OK;
}

ptg_status ptg_sampler_bench(ptg_ctx* c, const ptg_sampler_bench_cfg* cfg, double* v_plain, double* v_learned,
                             const ptg_sampler_bench_detail* detail, ptg_sampler_bench_stats* stats) {
    if (!c || !cfg) return set_err(PTG_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!c->mlp_ready) return set_err(PTG_ERR_INVALID_ARGUMENT, "no network: train or load one first");
    if (cfg->n == 0 || cfg->n > (1ull << 28)) return set_err(PTG_ERR_INVALID_ARGUMENT, "sample count out of range");
    if (!(cfg->margin >= 0.0f && cfg->margin < 10.0f)) return set_err(PTG_ERR_INVALID_ARGUMENT, "margin out of range");
    CUDA_TRY(cudaSetDevice(c->device));
    if (!c->tables_loaded) {
        ptg_status st = ptg_load_tables(c, nullptr);
        if (st != PTG_OK) return st;
    }
    unsigned long long n = cfg->n;
    float *dx = nullptr, *denv = nullptr;
    double *dv0 = nullptr, *dv1 = nullptr;
    unsigned *de0 = nullptr, *de1 = nullptr, *df = nullptr;
    int *ds0 = nullptr, *ds1 = nullptr;
    unsigned long long* ctr = nullptr;
    void* dpts = nullptr;
    auto cleanup = [&]() {
        cudaFree(dx), cudaFree(denv), cudaFree(dv0), cudaFree(dv1), cudaFree(de0), cudaFree(de1), cudaFree(df);
        cudaFree(ds0), cudaFree(ds1), cudaFree(ctr), cudaFree(dpts);
    };
    bool ok = cudaMalloc(&dx, 4 * MLP_IN * n) == cudaSuccess && cudaMalloc(&denv, 64 * n) == cudaSuccess &&
              cudaMalloc(&dv0, 8 * n) == cudaSuccess && cudaMalloc(&dv1, 8 * n) == cudaSuccess &&
              cudaMalloc(&de0, 4 * n) == cudaSuccess && cudaMalloc(&de1, 4 * n) == cudaSuccess &&
              cudaMalloc(&df, 4 * n) == cudaSuccess && cudaMalloc(&ds0, 4 * n) == cudaSuccess &&
              cudaMalloc(&ds1, 4 * n) == cudaSuccess && cudaMalloc(&ctr, 8) == cudaSuccess &&
              cudaMalloc(&dpts, sampler_point_bytes() * n) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        cleanup();
        return set_err(PTG_ERR_ALLOC, "sampler benchmark buffers");
    }
    cudaEvent_t e[5];
    for (auto& ev : e) cudaEventCreate(&ev);
    cudaStream_t s = c->stream;
    cudaError_t err = cudaSuccess;
    // the emissions' points (a, eta, n) and the network's inputs: shared
    cudaEventRecord(e[0], s);
    err = launch_sampler_features(c->lma_dev, n, cfg->seed, cfg->a_lo, cfg->a_hi, cfg->eta_lo, cfg->eta_hi, dx, dpts,
                                  s);
    cudaEventRecord(e[1], s);
    // plain: the reference's ceiling and rejection
    if (err == cudaSuccess)
        err = launch_sampler_run(c->lma_dev, n, cfg->seed, cfg->a_lo, cfg->a_hi, cfg->eta_lo, cfg->eta_hi, 0, nullptr,
                                 dpts, cfg->margin, ctr, dv0, de0, nullptr, ds0, s);
    cudaEventRecord(e[2], s);
    // learned: batched tensor-core inference, then sampling
    if (err == cudaSuccess) err = launch_mlp_infer(mlp_dev(c), c->mlp_packed, dx, n, denv, s);
    cudaEventRecord(e[3], s);
    if (err == cudaSuccess)
        err = launch_sampler_run(c->lma_dev, n, cfg->seed, cfg->a_lo, cfg->a_hi, cfg->eta_lo, cfg->eta_hi, 1, denv,
                                 dpts, cfg->margin, ctr, dv1, de1, df, ds1, s);
    cudaEventRecord(e[4], s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    std::vector<unsigned> ev0(n), ev1(n), fb(n);
    std::vector<int> st0(n), st1(n);
    if (err == cudaSuccess) {
        if (v_plain) cudaMemcpy(v_plain, dv0, 8 * n, cudaMemcpyDeviceToHost);
        if (v_learned) cudaMemcpy(v_learned, dv1, 8 * n, cudaMemcpyDeviceToHost);
        cudaMemcpy(ev0.data(), de0, 4 * n, cudaMemcpyDeviceToHost);
        cudaMemcpy(ev1.data(), de1, 4 * n, cudaMemcpyDeviceToHost);
        cudaMemcpy(fb.data(), df, 4 * n, cudaMemcpyDeviceToHost);
        cudaMemcpy(st0.data(), ds0, 4 * n, cudaMemcpyDeviceToHost);
        cudaMemcpy(st1.data(), ds1, 4 * n, cudaMemcpyDeviceToHost);
        if (detail) {
            if (detail->x) cudaMemcpy(detail->x, dx, 4 * MLP_IN * n, cudaMemcpyDeviceToHost);
            if (detail->env) cudaMemcpy(detail->env, denv, 64 * n, cudaMemcpyDeviceToHost);
            if (detail->status_plain) std::memcpy(detail->status_plain, st0.data(), 4 * n);
            if (detail->status_learned) std::memcpy(detail->status_learned, st1.data(), 4 * n);
            if (detail->evals_plain) std::memcpy(detail->evals_plain, ev0.data(), 4 * n);
            if (detail->evals_learned) std::memcpy(detail->evals_learned, ev1.data(), 4 * n);
            if (detail->fallback)
                for (unsigned long long q = 0; q < n; ++q) detail->fallback[q] = fb[q] & 3u;
        }
        err = cudaGetLastError();
    }
    float t_plain = 0, t_feat = 0, t_inf = 0, t_learn = 0;
    cudaEventElapsedTime(&t_feat, e[0], e[1]);
    cudaEventElapsedTime(&t_plain, e[1], e[2]);
    cudaEventElapsedTime(&t_inf, e[2], e[3]);
    cudaEventElapsedTime(&t_learn, e[3], e[4]);
    for (auto& ev : e) cudaEventDestroy(ev);
    cleanup();
    if (err != cudaSuccess) return set_err(PTG_ERR_CUDA, cudaGetErrorString(err));
    if (stats) {
        double s0 = 0, s1 = 0, proposals = 0, accepted = 0;
        unsigned long long nf = 0, nx = 0, ne0 = 0, ne1 = 0;
        for (unsigned long long i = 0; i < n; ++i) {
            unsigned kind = fb[i] & 3u;
            s0 += ev0[i], s1 += ev1[i];
            nf += (kind == 1u || kind == 3u) ? 1 : 0;
            nx += (kind == 2u || kind == 3u) ? 1 : 0;
            ne0 += st0[i] != 0 ? 1 : 0;
            ne1 += st1[i] != 0 ? 1 : 0;
            proposals += (double)(fb[i] >> 2);
            accepted += (st1[i] == 0 && (kind == 0u || kind == 2u)) ? 1.0 : 0.0;
        }
        stats->plain_ms = t_plain;
        stats->learned_ms = t_learn;
        stats->infer_ms = t_inf;
        stats->features_ms = t_feat;
        stats->acceptance = proposals > 0 ? accepted / proposals : 0.0;
        stats->plain_evals = s0 / (double)n;
        stats->learned_evals = s1 / (double)n;
        stats->fallbacks = nf;
        stats->exhausted = nx;
        stats->errors_plain = ne0;
        stats->errors_learned = ne1;
    }
    return PTG_OK;
}

// ------------------------------------------------ allocation-free batch ---
// ptg_collide_batch_noalloc(): the LCFA collision loop for callers that
// cannot allocate device memory.  Its working memory (wave counters, the
// primaries' initial momenta, per-shower counts, the pair-spectrum node
// constants and a fixed-size shower store) lives in one file-scope device
// array.  Host code never dereferences that array's name: the device
// address comes from cudaGetSymbolAddress() on every call.  Its waves run
// in slot order: putting a wave in order of laser phase needs sort buffers,
// and a batch of at most 4096 primaries gains little from it (the allocating
// path orders only waves of 2048 particles or more).  The results are the
// same either way, because each particle's random stream is fixed when it is
// created.
namespace {
constexpr unsigned long long NOALLOC_MAX_PRIMARIES = 4096;
constexpr unsigned long long NOALLOC_MAX_PARTICLES = 32768;  // shower store, primaries included
constexpr size_t noalloc_align(size_t b) { return (b + 255) & ~(size_t)255; }
constexpr size_t NOALLOC_STORE_BYTES = store_bytes(NOALLOC_MAX_PARTICLES);
constexpr size_t NOALLOC_OFF_COUNTERS = NOALLOC_STORE_BYTES;
constexpr size_t NOALLOC_OFF_INIT_U = NOALLOC_OFF_COUNTERS + noalloc_align(sizeof(Counters));
constexpr size_t NOALLOC_OFF_COUNTS = NOALLOC_OFF_INIT_U + noalloc_align(32 * NOALLOC_MAX_PRIMARIES);
constexpr size_t NOALLOC_OFF_GL = NOALLOC_OFF_COUNTS + noalloc_align(8 * NOALLOC_MAX_PRIMARIES);
constexpr size_t NOALLOC_BYTES = NOALLOC_OFF_GL + noalloc_align(sizeof(PairGL));
}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

// The pair-spectrum node constants, computed once per process on the host
// (they are the same on every device) and uploaded into the array by every
// call.
static std::mutex g_noalloc_mutex;
static PairGL g_noalloc_gl;
static bool g_noalloc_gl_ready = false;

// Every call, with the caller's device current: the array's device address
// in the current context (so that a context created after cudaDeviceReset,
// or another context made current on the same device, gets its own), and
// the constants uploaded on the call's stream ahead of its kernels.
static ptg_status noalloc_setup(cudaStream_t s, char** base) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || ptr == nullptr)
        return set_err(PTG_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (!g_noalloc_gl_ready) {
            CUDA_TRY(fill_pair_gl(&g_noalloc_gl));
            g_noalloc_gl_ready = true;
        }
    }
    CUDA_TRY(cudaMemcpyAsync((char*)ptr + NOALLOC_OFF_GL, &g_noalloc_gl, sizeof(PairGL), cudaMemcpyHostToDevice, s));
    *base = (char*)ptr;
    return PTG_OK;
}

__global__ void k_noalloc_reset(Counters* c, unsigned long long n) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        *c = Counters{};
        c->n_total = n;
    }
}

static cudaError_t noalloc_wave(const WaveArgs& a, int grid_max, cudaStream_t s) {
    unsigned long long n = a.hi - a.lo;
    unsigned long long need = (n + 127) / 128;
    int grid = (unsigned long long)grid_max > need ? (int)need : grid_max;
    if (grid < 1) grid = 1;
    return launch_wave_lcfa(a.f.model, grid, 128, s, a);
}

ptg_status ptg_collide_batch_noalloc(const ptg_laser_desc* laser, const ptg_collide_options* o,
                                     const ptg_particles* d_primaries, uint64_t seed, uint64_t id_base,
                                     ptg_particles* d_out, size_t out_capacity, void* stream, ptg_run_stats* stats) {
    ptg_status st = check_laser(laser);
    if (st != PTG_OK) return st;
    if (!o || !d_primaries || !d_out) return set_err(PTG_ERR_INVALID_ARGUMENT, "NULL argument");
    if (laser->model != PTG_FAST_PLANE_WAVE && laser->model != PTG_FAST_FOCUSED_LASER)
        return set_err(PTG_ERR_UNSUPPORTED, "the allocation-free entry point covers the LCFA field models only");
    if (!(o->rate_increase >= 1.0)) return set_err(PTG_ERR_INVALID_ARGUMENT, "increase in pair creation rate must be >= 1.0");
    if (o->rate_increase > 1.0 && o->multiplicity >= 0)
        return set_err(PTG_ERR_INVALID_ARGUMENT, "event biasing is incompatible with multiplicity selection");
    if (d_primaries->n == 0) {
        // no primaries: an empty shower, as ptg_collide_batch_device gives
        d_out->n = 0;
        if (stats) std::memset(stats, 0, sizeof(*stats));
        return PTG_OK;
    }
    if (!d_primaries->species || !d_primaries->r || !d_primaries->u)
        return set_err(PTG_ERR_INVALID_ARGUMENT, "primaries need species, r and u");
    if (d_primaries->n > NOALLOC_MAX_PRIMARIES)
        return set_err(PTG_ERR_INVALID_ARGUMENT, "the allocation-free entry point takes at most " +
                                                     std::to_string(NOALLOC_MAX_PRIMARIES) + " primaries per call, got " +
                                                     std::to_string(d_primaries->n));
    if (!d_out->species || !d_out->r || !d_out->u || !d_out->r0 || !d_out->u0 || !d_out->pol || !d_out->weight ||
        !d_out->payload || !d_out->parent_chi || !d_out->interaction_count || !d_out->work || !d_out->id ||
        !d_out->parent_id || !d_out->primary || !d_out->stream || !d_out->generation || !d_out->flags || !d_out->status)
        return set_err(PTG_ERR_INVALID_ARGUMENT, "every output array must be a device buffer of out_capacity rows");
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    cudaStream_t s = (cudaStream_t)stream;
    char* base = nullptr;
    st = noalloc_setup(s, &base);
    if (st != PTG_OK) return st;
    int sms = 0, per_sm = 0;
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));

    Store store;
    carve_store(&store, base, NOALLOC_MAX_PARTICLES);
    Counters* counters = (Counters*)(base + NOALLOC_OFF_COUNTERS);
    double* init_u = (double*)(base + NOALLOC_OFF_INIT_U);
    unsigned long long* shower_count = (unsigned long long*)(base + NOALLOC_OFF_COUNTS);
    const PairGL* gl = (const PairGL*)(base + NOALLOC_OFF_GL);

    unsigned long long n = d_primaries->n;
    double dt_max;
    WaveArgs a{};
    a.f = make_field(*laser, &dt_max);
    fill_step_options(*o, &a.o);
    a.o.dt = dt_max * o->dt_multiplier;
    a.s = store;
    a.c = counters;
    a.gl = gl;
    a.lma = nullptr;
    a.seed = seed;
    a.n_primaries = n;
    a.id_base = id_base;
    const void* kern = wave_kernel_lcfa(laser->model);
    CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, 0));
    int grid_max = (per_sm > 0 ? per_sm : 1) * sms;

    // the array keeps the previous call's contents: reset the counters
    k_noalloc_reset<<<1, 32, 0, s>>>(counters, n);
    CUDA_TRY(cudaGetLastError());
    if (n > 0) {
        k_load_primaries<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(store, *d_primaries, n, id_base, init_u, shower_count);
        CUDA_TRY(cudaGetLastError());
    }
    Counters h{};
    unsigned long long lo = 0, hi = n;
    uint32_t waves = 0;
    while (lo < hi) {
        a.lo = lo;
        a.hi = hi;
        CUDA_TRY(cudaMemsetAsync(&counters->next, 0, 8, s));
        CUDA_TRY(noalloc_wave(a, grid_max, s));
        ++waves;
        CUDA_TRY(cudaMemcpyAsync(&h, counters, sizeof(Counters), cudaMemcpyDeviceToHost, s));
        CUDA_TRY(cudaStreamSynchronize(s));
        if (h.overflow)
            return set_err(PTG_ERR_QUEUE_OVERFLOW, "the shower outgrew the allocation-free store (" +
                                                       std::to_string(NOALLOC_MAX_PARTICLES) + " particles)");
        lo = hi;
        hi = h.n_total;
    }
    unsigned long long total = hi;
    FilterArgs fa{};
    fa.s = store;
    fa.init_u = init_u;
    fa.shower_count = shower_count;
    fa.n = total;
    fa.min_energy = o->min_energy;
    fa.cos_max_angle = std::cos(o->max_angle);
    fa.discard_bg_e = o->discard_bg_e;
    fa.discard_bg_ph = o->discard_bg_ph;
    fa.multiplicity = o->multiplicity;
    unsigned blocks = (unsigned)((total + 255) / 256);
    if (blocks == 0) blocks = 1;
    if (o->multiplicity >= 0) {
        k_filter_count<<<blocks, 256, 0, s>>>(fa);
        CUDA_TRY(cudaGetLastError());
    }
    k_compact<<<blocks, 256, 0, s>>>(fa, counters, *d_out, out_capacity);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(&h, counters, sizeof(Counters), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->n_primaries = n;
        stats->n_out = h.n_out;
        stats->n_created = total;
        stats->lepton_steps = h.lepton_steps;
        stats->photon_steps = h.photon_steps;
        stats->emissions = h.emissions;
        stats->pair_events = h.pair_events;
        stats->rejections = h.rejections;
        stats->particle_errors = h.errors;
        stats->waves = waves;
        stats->max_steps = h.max_steps;
        stats->free_steps = h.free_steps;
        stats->drift_steps = h.drift_steps;
    }
    if (h.n_out > out_capacity)
        return set_err(PTG_ERR_QUEUE_OVERFLOW, "the output needs " + std::to_string(h.n_out) + " rows, out_capacity is " +
                                                   std::to_string(out_capacity));
    d_out->n = h.n_out;
    return PTG_OK;
}
