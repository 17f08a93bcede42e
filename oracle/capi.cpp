// Oracle (test infrastructure only): extern "C" entry points for the tests,
// smoke() and bench.py's CPU-baseline leg.  Built into
// oracle/_build/liboracle.so; nothing in the product library links it.
#include <atomic>
#include <string>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "fields.h"
#include "lma.h"
#include "physics.h"

using namespace orc;

static V4 v4(const double* p) { return V4(p[0], p[1], p[2], p[3]); }
static V3 v3(const double* p) { return V3(p[0], p[1], p[2]); }
static void put4(double* p, const V4& v) { p[0] = v.t, p[1] = v.x, p[2] = v.y, p[3] = v.z; }
static void put3(double* p, const V3& v) { p[0] = v.x, p[1] = v.y, p[2] = v.z; }

extern "C" {

double orc_lcfa_photon_rate(double chi, double gamma) { return lcfa_photon_rate(chi, gamma); }
double orc_lcfa_classical_rate(double chi, double gamma) { return lcfa_classical_rate(chi, gamma); }

void orc_lcfa_photon_sample(double chi, double gamma, double r1, double r2, double r3, double* omega, double* theta,
                            double* cphi) {
    bool has;
    lcfa_photon_sample(chi, gamma, r1, r2, r3, omega, &has, theta, cphi);
    if (!has) *theta = -1.0;
}

void orc_lcfa_stokes(const double* k, double chi, double gamma, const double* v, const double* w, double* out) {
    Stokes s = lcfa_stokes_parameters(v4(k), chi, gamma, v3(v), v3(w));
    out[0] = s.i, out[1] = s.q, out[2] = s.u, out[3] = s.v;
}

double orc_gaunt_factor(double chi) { return gaunt_factor(chi); }

void orc_lcfa_pair_t(double chi, double* par, double* perp) { lcfa_auxiliary_t(chi, par, perp); }

double orc_lcfa_pair_probability(const double* ell, const double* sv, double chi, const double* a_perp, double dt,
                                 double* sv_new) {
    Stokes out;
    double p = lcfa_pair_probability(v4(ell), Stokes(sv[0], sv[1], sv[2], sv[3]), chi, v3(a_perp), dt, &out);
    sv_new[0] = out.i, sv_new[1] = out.q, sv_new[2] = out.u, sv_new[3] = out.v;
    return p;
}

double orc_lcfa_pair_spectrum(double s, double chi, double sv1) { return lcfa_pair_spectrum(s, chi, sv1); }
double orc_lcfa_pair_spectrum_ceiling(double chi, double sv1) { return lcfa_pair_spectrum_ceiling(chi, sv1); }
double orc_lcfa_pair_angular_spectrum(double y, double s, double chi, double sv1) {
    return lcfa_pair_angular_spectrum(y, s, chi, sv1);
}
double orc_lcfa_pair_angular_spectrum_ceiling(double s, double chi, double sv1) {
    return lcfa_pair_angular_spectrum_ceiling(s, chi, sv1);
}

// Samples one LCFA pair event with the stream (seed, stream, step).
int orc_lcfa_pair_sample(const double* ell, const double* sv, double chi, const double* a_perp, uint64_t seed,
                         uint64_t stream, uint32_t step, double* out5) {
    DrawStream rng;
    rng.seed = seed;
    rng.stream = stream;
    rng.begin_step(step);
    return lcfa_pair_sample(v4(ell), Stokes(sv[0], sv[1], sv[2], sv[3]), chi, v3(a_perp), rng, &out5[0], &out5[1],
                            &out5[2], &out5[3], &out5[4])
               ? 0
               : PTG_ERR_REJECTION_CAP;
}

double orc_airy_ai(double x) {
    bool ok;
    double v = airy_ai(x, &ok);
    return ok ? v : NAN;
}
double orc_airy_ai_prime(double x) {
    bool ok;
    double v = airy_ai_prime(x, &ok);
    return ok ? v : NAN;
}
double orc_bessel_k13(double x) {
    bool ok;
    double v = bessel_k_1_3(x, &ok);
    return ok ? v : NAN;
}
double orc_bessel_k23(double x) {
    bool ok;
    double v = bessel_k_2_3(x, &ok);
    return ok ? v : NAN;
}

double orc_pwmci_evaluate(const double* tbl, int n, int ext, double x, int* ok) {
    bool b;
    double v = Pwmci(tbl, n, ext != 0).evaluate(x, &b);
    *ok = b;
    return v;
}
double orc_pwmci_invert(const double* tbl, int n, int ext, double f, int* ok) {
    bool b;
    double v = Pwmci(tbl, n, ext != 0).invert(f, &b);
    *ok = b;
    return v;
}

void orc_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
    uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
    philox4x32_10(c, key[0], key[1]);
    std::memcpy(out, c, sizeof(c));
}

void orc_draws(uint64_t seed, uint64_t stream, uint32_t step, int n, double* out) {
    DrawStream rng;
    rng.seed = seed;
    rng.stream = stream;
    rng.begin_step(step);
    for (int k = 0; k < n; ++k) out[k] = rng.next();
}

uint64_t orc_primary_stream(uint64_t idx) { return primary_stream(idx); }
uint64_t orc_child_stream(uint64_t parent, uint32_t step, uint32_t slot) { return child_stream(parent, step, slot); }

double orc_max_timestep(const ptg_laser_desc* d) { return Laser(*d).max_timestep(); }
double orc_initial_z(const ptg_laser_desc* d) { return Laser(*d).ideal_initial_z(); }
int orc_contains(const ptg_laser_desc* d, const double* r) { return Laser(*d).contains(v4(r)); }

void orc_fields(const ptg_laser_desc* d, const double* r, double* E, double* B, double* a) {
    V3 e, b;
    Laser(*d).fields(v4(r), &e, &b, a);
    put3(E, e);
    put3(B, b);
}

double orc_a_sqd(const ptg_laser_desc* d, const double* r) { return Laser(*d).a_sqd(v4(r)); }

void orc_push(const ptg_laser_desc* d, const double* r, const double* u, double rqm, double dt, int eqn, double* r_out,
              double* u_out, double* dt_out, double* work) {
    V4 ro, uo;
    Laser(*d).push(v4(r), v4(u), rqm, dt, eqn, &ro, &uo, dt_out, work);
    put4(r_out, ro);
    put4(u_out, uo);
}

// Repeated pushes of n particles (classical trajectories, emission off).
void orc_push_steps(const ptg_laser_desc* d, size_t n, double* r, double* u, double rqm, double dt, int eqn,
                    int nsteps, double* work) {
    Laser L(*d);
    for (size_t i = 0; i < n; ++i) {
        V4 rr = v4(r + 4 * i), uu = v4(u + 4 * i);
        double w = 0.0;
        for (int s = 0; s < nsteps; ++s) {
            double dto, dw;
            L.push(rr, uu, rqm, dt, eqn, &rr, &uu, &dto, &dw);
            w += dw;
        }
        put4(r + 4 * i, rr);
        put4(u + 4 * i, uu);
        if (work) work[i] = w;
    }
}

int orc_load_tables(const char* dir) {
    std::string err;
    return load_lma_tables(dir, &err) ? 0 : 1;
}
int orc_has_lp_mid_cdf() { return g_lma.bw_lp_mid_cdf != nullptr; }
int orc_has_cp_cdf(void) { return g_lma.nlc_cp_cdf != nullptr; }

double orc_bessel_j(double x, int n) { return bessel_j(x, n); }
double orc_bessel_triple_j(int n, double x) { return bessel_triple_j_mid(n, x); }
double orc_bessel_j_asymptotic(int n, double x) { return bessel_j_asymptotic(n, x); }
void orc_bessel_j_pm(double x, int n, double* out3) { bessel_j_pm(x, n, &out3[0], &out3[1], &out3[2]); }

double orc_cp_diff_partial_rate(int n, double a, double eta, double v) { return cp_diff_partial_rate(n, a, eta, v); }
double orc_cp_ceiling(int n, double a, double eta) { return cp_ceiling_diff_partial_rate(n, a, eta); }
double orc_cp_partial_rate(int n, double a, double eta) { return cp_partial_rate(n, a, eta); }
double orc_cp_rate(double a, double eta) {
    double r;
    return cp_rate(a, eta, &r) ? r : NAN;
}
int orc_cp_invert(double a, double eta, double frac) { return cp_invert(a, eta, frac); }

// One CP emission sample with the stream (seed, stream, step): n, s, theta, Stokes[4]
int orc_cp_sample(double a, double eta, uint64_t seed, uint64_t stream, uint32_t step, double* out7) {
    DrawStream rng;
    rng.seed = seed;
    rng.stream = stream;
    rng.begin_step(step);
    int n;
    double s, th;
    Stokes sv;
    uint64_t rej = 0;
    int st = cp_sample(a, eta, rng, &n, &s, &th, &sv, &rej);
    out7[0] = n, out7[1] = s, out7[2] = th, out7[3] = sv.i, out7[4] = sv.q, out7[5] = sv.u, out7[6] = sv.v;
    return st;
}

// LMA emission (nonlinear_compton::generate) for given k, q, with a stream
int orc_nlc_generate(const double* k, const double* q, int pol, double pol_angle, uint64_t seed, uint64_t stream,
                     uint32_t step, double* out9) {
    DrawStream rng;
    rng.seed = seed;
    rng.stream = stream;
    rng.begin_step(step);
    int n;
    V4 kp;
    Stokes sv;
    uint64_t rej = 0;
    int st = nlc_generate(v4(k), v4(q), pol, pol_angle, false, rng, &n, &kp, &sv, &rej);
    out9[0] = n;
    put4(out9 + 1, kp);
    out9[5] = sv.i, out9[6] = sv.q, out9[7] = sv.u, out9[8] = sv.v;
    return st;
}

double orc_nlc_probability(const double* k, const double* q, double dt, int pol) {
    double p;
    return nlc_probability(v4(k), v4(q), dt, pol, false, &p) ? p : NAN;
}

void orc_cp_pair_integrate(int n, double a, double eta, double* out2) { cp_pair_integrate(n, a, eta, &out2[0], &out2[1]); }
void orc_cp_pair_by_summation(double a, double eta, double* out2) { cp_pair_by_summation(a, eta, out2); }
int orc_cp_pair_by_lookup(double a, double eta, double* out2) { return cp_pair_by_lookup(a, eta, out2) ? 0 : 1; }
int orc_cp_pair_rates(double a, double eta, double* out2) { return cp_pair_rates(a, eta, out2) ? 0 : 1; }

// LMA pair probability (pair_creation::probability) and one generated positron
double orc_bw_probability(const double* ell, const double* sv, const double* k, double a, double dt, int pol,
                          double pol_angle, double* sv_out) {
    double p;
    Stokes out;
    if (!bw_probability(v4(ell), Stokes(sv[0], sv[1], sv[2], sv[3]), v4(k), a, dt, pol, pol_angle, &p, &out)) return NAN;
    sv_out[0] = out.i, sv_out[1] = out.q, sv_out[2] = out.u, sv_out[3] = out.v;
    return p;
}

int orc_bw_generate(const double* ell, const double* sv, const double* k, double a, int pol, double pol_angle,
                    uint64_t seed, uint64_t stream, uint32_t step, double* out5) {
    DrawStream rng;
    rng.seed = seed;
    rng.stream = stream;
    rng.begin_step(step);
    int n;
    V4 q;
    uint64_t rej = 0;
    int st = bw_generate(v4(ell), Stokes(sv[0], sv[1], sv[2], sv[3]), v4(k), a, pol, pol_angle, rng, &n, &q, &rej);
    out5[0] = n;
    put4(out5 + 1, q);
    return st;
}

double orc_double_bessel_at(int n, double x_max, double y_max, double x, double y) {
    return double_bessel_at(n, x_max, y_max, x, y);
}
double orc_double_bessel_evaluate(int n, double x, double y) { return double_bessel_evaluate(n, x, y); }
double orc_double_bessel_spa(int n, double x, double y) { return double_bessel_spa(n, x, y); }
double orc_lp_ceiling(int n, double a, double eta) { return lp_ceiling_at(n, a, eta); }
void orc_lp_partial_rate(int n, double a, double eta, double* out2) { lp_partial_rate(n, a, eta, &out2[0], &out2[1]); }
int orc_lp_sum_limit(double a, double eta) { return lp_sum_limit(a, eta); }
double orc_lp_rate(double a, double eta) {
    double r;
    return lp_rate(a, eta, &r) ? r : NAN;
}
int orc_lp_harmonic_index(double a, double eta, double frac) { return lp_harmonic_index(a, eta, frac); }
int orc_lp_sample(double a, double eta, uint64_t seed, uint64_t stream, uint32_t step, double* out7) {
    DrawStream rng;
    rng.seed = seed;
    rng.stream = stream;
    rng.begin_step(step);
    int n;
    double s, th;
    Stokes sv;
    uint64_t rej = 0;
    int st = lp_sample(a, eta, rng, &n, &s, &th, &sv, &rej);
    out7[0] = n, out7[1] = s, out7[2] = th, out7[3] = sv.i, out7[4] = sv.q, out7[5] = sv.u, out7[6] = sv.v;
    return st;
}

void orc_lp_pair_rates(double a, double eta, double* out2) {
    if (!lp_pair_rates(a, eta, out2)) out2[0] = out2[1] = NAN;
}
void orc_lp_pair_dd_rate(int n, double a, double eta, double s, double theta, double* out2) {
    lp_pair_dd_rate(n, a, eta, s, theta, out2);
}
void orc_lp_pair_partial_rate(int n, double a, double eta, double* out2) { lp_pair_partial_rate(n, a, eta, out2); }
void orc_lp_pair_by_summation(double a, double eta, double* cdf48) { lp_pair_by_summation(a, eta, cdf48); }
int orc_lp_pair_sample(double a, double eta, double sv1, double sv2, uint64_t seed, uint64_t stream, uint32_t step,
                       double* out3) {
    DrawStream rng;
    rng.seed = seed;
    rng.stream = stream;
    rng.begin_step(step);
    int n = 0;
    double s = 0.0, th = 0.0;
    uint64_t rej = 0;
    int st = lp_pair_sample(a, eta, sv1, sv2, rng, &n, &s, &th, &rej);
    out3[0] = n, out3[1] = s, out3[2] = th;
    return st;
}

double orc_cp_cl_integrated(int n, double a) { return cp_cl_integrated(n, a); }
double orc_lp_cl_partial_rate(int n, double a) { return lp_cl_partial_rate(n, a); }
double orc_nlc_classical_rate(double a, double eta, int pol) {
    double r;
    bool ok = pol == 1 ? cp_classical_rate(a, eta, &r) : lp_classical_rate(a, eta, &r);
    return ok ? r : NAN;
}
int orc_nlc_classical_sample(double a, double eta, int pol, uint64_t seed, uint64_t stream, uint32_t step,
                             double* out7) {
    DrawStream rng;
    rng.seed = seed;
    rng.stream = stream;
    rng.begin_step(step);
    int n = 0;
    double s = 0.0, th = 0.0;
    Stokes sv;
    uint64_t rej = 0;
    int st = pol == 1 ? cp_classical_sample(a, eta, rng, &n, &s, &th, &sv, &rej)
                      : lp_classical_sample(a, eta, rng, &n, &s, &th, &sv, &rej);
    out7[0] = n, out7[1] = s, out7[2] = th, out7[3] = sv.i, out7[4] = sv.q, out7[5] = sv.u, out7[6] = sv.v;
    return st;
}

struct OrcResult {
    std::vector<OracleParticle> parts;
    OracleStats stats;
};

// main.rs:1118-1135 over a batch; threads work on disjoint primaries.
void* orc_collide_run(const ptg_laser_desc* d, const ptg_collide_options* o, const ptg_particles* in, uint64_t seed,
                      uint64_t id_base, int nthreads) {
    Laser L(*d);
    size_t n = in->n;
    std::vector<std::vector<OracleParticle>> showers(n);
    std::vector<OracleStats> tstats(nthreads > 0 ? nthreads : 1);
    std::vector<uint64_t> created(n, 0);
    std::atomic<size_t> next(0);
    const uint64_t LOCAL = 1ull << 62;
    auto work = [&](int tid) {
        OracleStats& st = tstats[tid];
        while (true) {
            size_t i = next.fetch_add(1);
            if (i >= n) break;
            OracleParticle p{};
            p.species = in->species[i];
            p.r = v4(in->r + 4 * i);
            p.u = v4(in->u + 4 * i);
            p.r0 = in->r0 ? v4(in->r0 + 4 * i) : p.r;
            p.u0 = in->u0 ? v4(in->u0 + 4 * i) : (p.species == PTG_PHOTON ? V4(0, 0, 0, 0) : V4(1, 0, 0, 0));
            p.pol = in->pol ? Stokes(in->pol[4 * i], in->pol[4 * i + 1], in->pol[4 * i + 2], in->pol[4 * i + 3])
                            : Stokes::unpolarized();
            p.weight = in->weight ? in->weight[i] : 1.0;
            p.id = in->id ? in->id[i] : i;
            p.parent_id = in->parent_id ? in->parent_id[i] : p.id;
            p.primary = i;
            p.stream = primary_stream(id_base + i);
            uint64_t cur = LOCAL;
            uint64_t before = st.created;
            collide(L, *o, p, seed, &cur, showers[i], st);
            created[i] = st.created - before;
        }
    };
    int nt = nthreads > 0 ? nthreads : 1;
    std::vector<std::thread> th;
    for (int t = 1; t < nt; ++t) th.emplace_back(work, t);
    work(0);
    for (auto& t : th) t.join();
    OrcResult* res = new OrcResult;
    uint64_t off = id_base;
    for (size_t i = 0; i < n; ++i) {
        for (auto& p : showers[i]) {
            if (p.id >= LOCAL) p.id = p.id - LOCAL + off;
            if (p.parent_id >= LOCAL) p.parent_id = p.parent_id - LOCAL + off;
            res->parts.push_back(p);
        }
        off += created[i];
    }
    for (auto& s : tstats) {
        res->stats.lepton_steps += s.lepton_steps;
        res->stats.photon_steps += s.photon_steps;
        res->stats.emissions += s.emissions;
        res->stats.pair_events += s.pair_events;
        res->stats.rejections += s.rejections;
        res->stats.created += s.created;
    }
    return res;
}

size_t orc_result_size(void* h) { return ((OrcResult*)h)->parts.size(); }

void orc_result_stats(void* h, ptg_run_stats* st) {
    OrcResult* r = (OrcResult*)h;
    std::memset(st, 0, sizeof(*st));
    st->n_out = r->parts.size();
    st->n_created = r->stats.created;
    st->lepton_steps = r->stats.lepton_steps;
    st->photon_steps = r->stats.photon_steps;
    st->emissions = r->stats.emissions;
    st->pair_events = r->stats.pair_events;
    st->rejections = r->stats.rejections;
    for (auto& p : r->parts)
        if (p.status != 0) st->particle_errors++;
}

// Copies into caller-allocated arrays of at least orc_result_size() rows.
void orc_result_copy(void* h, ptg_particles* o) {
    OrcResult* r = (OrcResult*)h;
    size_t n = r->parts.size();
    for (size_t i = 0; i < n; ++i) {
        const OracleParticle& p = r->parts[i];
        if (o->species) o->species[i] = p.species;
        if (o->r) put4(o->r + 4 * i, p.r);
        if (o->u) put4(o->u + 4 * i, p.u);
        if (o->r0) put4(o->r0 + 4 * i, p.r0);
        if (o->u0) put4(o->u0 + 4 * i, p.u0);
        if (o->pol) {
            o->pol[4 * i] = p.pol.i, o->pol[4 * i + 1] = p.pol.q, o->pol[4 * i + 2] = p.pol.u;
            o->pol[4 * i + 3] = p.pol.v;
        }
        if (o->weight) o->weight[i] = p.weight;
        if (o->payload) o->payload[i] = p.payload;
        if (o->parent_chi) o->parent_chi[i] = p.parent_chi;
        if (o->interaction_count) o->interaction_count[i] = p.interaction_count;
        if (o->work) o->work[i] = p.work;
        if (o->id) o->id[i] = p.id;
        if (o->parent_id) o->parent_id[i] = p.parent_id;
        if (o->primary) o->primary[i] = p.primary;
        if (o->stream) o->stream[i] = p.stream;
        if (o->generation) o->generation[i] = p.generation;
        if (o->flags) o->flags[i] = p.flags;
        if (o->status) o->status[i] = p.status;
    }
    o->n = n;
}

void orc_result_free(void* h) { delete (OrcResult*)h; }

}  // extern "C"
