// Oracle (test infrastructure only): see fields.h.
#include "fields.h"

#include <algorithm>
#include <cmath>
#include <complex>

#include "lma.h"

namespace orc {

using cplx = std::complex<double>;

static inline double sq(double x) { return x * x; }
static inline double powi(double a, int b) {
    bool recip = b < 0;
    unsigned n = recip ? (unsigned)(-b) : (unsigned)b;
    double r = 1.0;
    while (true) {
        if (n & 1u) r *= a;
        n >>= 1;
        if (n == 0) break;
        a *= a;
    }
    return recip ? 1.0 / r : r;
}
constexpr double LN_2 = 0.693147180559945309417232121458176568;
constexpr double FRAC_PI_2 = 1.57079632679489661923132169163975144;

Laser::Laser(const ptg_laser_desc& desc) : d(desc) {
    double k = 2.0 * PI / d.wavelength;
    wavevector = V4(k, 0.0, 0.0, k);
    duration = d.n_cycles * d.wavelength / SPEED_OF_LIGHT;
    // PlaneWave::new keeps pol_angle as given; the LCFA models zero it for CP
    // (fast_plane_wave.rs:31-34, fast_focused_laser.rs:32-35).
    if (lcfa() && d.polarization == PTG_POL_CIRCULAR) d.pol_angle = 0.0;
    bandwidth = 0.0;
    if (!lcfa() && d.finite_bandwidth) {
        // plane_wave.rs:49-61, focused_laser.rs:55-67
        double nc = n_cycles();
        double n_fwhm = (d.envelope == PTG_ENV_COS2) ? 0.36405666377387671305 * nc : nc;
        bandwidth = std::sqrt(0.5 * LN_2) / (PI * n_fwhm);
    }
}

double Laser::n_cycles() const {
    if (d.model == PTG_FOCUSED_LASER || d.model == PTG_FAST_FOCUSED_LASER)
        return SPEED_OF_LIGHT * duration * wavevector.t / (2.0 * PI);  // focused_laser.rs:50-53
    return d.n_cycles;
}

double Laser::max_timestep() const {
    switch (d.model) {
        case PTG_PLANE_WAVE:  // plane_wave.rs:175-181
            return (d.envelope == PTG_ENV_FLATTOP ? 0.2 : 1.0) / (SPEED_OF_LIGHT * wavevector.t);
        case PTG_FOCUSED_LASER:  // focused_laser.rs:183-189
            return (d.envelope == PTG_ENV_FLATTOP ? 0.2 : 1.0) / omega();
        case PTG_FAST_PLANE_WAVE: {  // fast_plane_wave.rs:89-98
            double chirp = 1.0 + 2.0 * d.chirp_b * PI * d.n_cycles;
            double dt = 1.0 / (SPEED_OF_LIGHT * wavevector.t * chirp);
            double m = std::min(std::sqrt(3.0) / (5.0 * ALPHA_FINE * d.a0), 0.1);
            return dt * m;
        }
        default: {  // fast_focused_laser.rs:155-159
            double dt = 1.0 / omega();
            double m = std::min(std::sqrt(3.0) / (5.0 * ALPHA_FINE * d.a0), 0.1);
            return dt * m;
        }
    }
}

bool Laser::contains(const V4& r) const {
    double phase = wavevector * r;
    double nc = n_cycles();
    double max_phase;
    switch (d.envelope) {
        case PTG_ENV_COS2: max_phase = PI * nc; break;
        case PTG_ENV_FLATTOP: max_phase = PI * (nc + 1.0); break;
        default: max_phase = 6.0 * PI * nc; break;
    }
    return phase < max_phase;
}

double Laser::ideal_initial_z() const {
    double wavelength = 2.0 * PI / wavevector.t;
    double nc = n_cycles();
    switch (d.envelope) {
        case PTG_ENV_COS2: return 0.5 * wavelength * nc;
        case PTG_ENV_FLATTOP: return 0.5 * wavelength * (nc + 1.0);
        default: return 2.0 * wavelength * nc;
    }
}

// fast_focused_laser.rs:59-111 (Salamin, Appl. Phys. B 86, 319 (2007))
void Laser::ffl_beam(const V4& r_in, V3* reE, V3* imE, V3* reB, V3* imB) const {
    V4 r = r_in.rotate_around_z(-d.pol_angle);
    double zr = 0.5 * wavevector.t * sq(d.waist);
    double x = r.x / d.waist, y = r.y / d.waist, z = r.z / zr;
    double rho = std::hypot(x, y);
    double e = d.waist / zr;
    const cplx i(0.0, 1.0);
    cplx f = i / (z + i);
    cplx pre = f * std::exp(-f * powi(rho, 2) + i * (wavevector * r + 0.0));
    double rho2 = powi(rho, 2), rho4 = powi(rho, 4), rho6 = powi(rho, 6), rho8 = powi(rho, 8);
    cplx f2 = f * f, f3 = f * f * f, f4 = f * f * f * f;
    cplx Ex = -i * pre *
              (1.0 + powi(e, 2) * f * f * (x * x - f * rho4 / 4.0) +
               powi(e, 4) * f * f *
                   (1.0 / 8.0 - f * rho2 / 4.0 + f * f * (powi(x * rho, 2) - rho4 / 16.0) +
                    f3 * rho4 * (-x * x - 0.5 * rho2) / 4.0 + f4 * rho8 / 32.0));
    cplx Ey = -i * pre * (powi(e, 2) * f * f * x * y + powi(e, 4) * x * y * std::pow(f, 4.0) * rho2 * (1.0 - f * rho2 / 4.0));
    cplx Ez = pre * (e * f * x + powi(e, 3) * f * f * x * (-0.5 + f * rho2 - f * f * rho4 / 4.0));
    cplx Bx(0.0, 0.0);
    cplx By = -i * pre *
              (1.0 + powi(e, 2) * f * f * rho2 * (1.0 - f * rho2 / 2.0) / 2.0 +
               powi(e, 4) * f * f * (-1.0 + 2.0 * f * rho2 + 2.5 * f2 * rho4 - 2.0 * f3 * rho6 + 0.25 * f4 * rho8) / 8.0);
    cplx Bz = pre * (e * f * y + powi(e, 3) * f * f * y * (1.0 + f * rho2 - f * f * rho4 / 2.0) / 2.0);
    double E0 = ELECTRON_MASS * SPEED_OF_LIGHT * omega() * d.a0 / ELEMENTARY_CHARGE;
    double B0 = E0 / SPEED_OF_LIGHT;
    *reE = (E0 * V3(Ex.real(), Ey.real(), Ez.real())).rotate_around_z(d.pol_angle);
    *imE = (E0 * V3(Ex.imag(), Ey.imag(), Ez.imag())).rotate_around_z(d.pol_angle);
    *reB = (B0 * V3(Bx.real(), By.real(), Bz.real())).rotate_around_z(d.pol_angle);
    *imB = (B0 * V3(Bx.imag(), By.imag(), Bz.imag())).rotate_around_z(d.pol_angle);
}

// fast_focused_laser.rs:123-151
void Laser::ffl_envelope(double phase, double* f, double* df) const {
    double nc = n_cycles();
    switch (d.envelope) {
        case PTG_ENV_COS2:
            if (std::fabs(phase) < PI * nc) {
                double env = powi(std::cos(phase / (2.0 * nc)), 2);
                *f = env;
                *df = -1.0 * std::tan(phase / (2.0 * nc)) * env / nc;
            } else {
                *f = 0.0, *df = 0.0;
            }
            return;
        case PTG_ENV_FLATTOP:
            if (std::fabs(phase) > PI * (nc + 1.0)) {
                *f = 0.0, *df = 0.0;
            } else if (std::fabs(phase) > PI * (nc - 1.0)) {
                double arg = 0.25 * (std::fabs(phase) - (nc - 1.0) * PI);
                *f = powi(std::cos(arg), 2);
                *df = -0.25 * signum(phase) * std::sin(2.0 * arg);
            } else {
                *f = 1.0, *df = 0.0;
            }
            return;
        default: {
            double tau = omega() * duration;
            double env = std::exp(-2.0 * LN_2 * powi(phase, 2) / powi(tau, 2));
            *f = env;
            *df = -4.0 * LN_2 * phase * env / powi(tau, 2);
        }
    }
}

void Laser::fields(const V4& r, V3* E_out, V3* B_out, double* a_out) const {
    if (d.model == PTG_FAST_PLANE_WAVE) {
        // fast_plane_wave.rs:121-195 (without the compensating-chirp feature)
        double delta = d.polarization == PTG_POL_CIRCULAR ? 1.0 : 0.0;
        double phi = wavevector * r;
        double psi = phi * (1.0 + d.chirp_b * phi);
        double dpsi = 1.0 + 2.0 * d.chirp_b * phi;
        double nc = d.n_cycles;
        double f, df;
        switch (d.envelope) {
            case PTG_ENV_COS2:
                if (std::fabs(phi) < nc * PI) {
                    f = powi(std::cos(phi / (2.0 * nc)), 2);
                    df = -std::sin(phi / nc) / (2.0 * nc);
                } else {
                    f = 0.0, df = 0.0;
                }
                break;
            case PTG_ENV_FLATTOP:
                if (std::fabs(phi) > PI * (nc + 1.0)) {
                    f = 0.0, df = 0.0;
                } else if (std::fabs(phi) > PI * (nc - 1.0)) {
                    double arg = 0.25 * (std::fabs(phi) - (nc - 1.0) * PI);
                    f = powi(std::cos(arg), 2);
                    df = -signum(phi) * 0.25 * std::sin(2.0 * arg);
                } else {
                    f = 1.0, df = 0.0;
                }
                break;
            default: {
                double arg = -0.5 * powi(phi / (PI * nc), 2);
                f = std::exp2(arg);
                df = -LN_2 * phi * std::exp2(arg) / powi(PI * nc, 2);
            }
        }
        double dax = std::sin(psi) * df + std::cos(psi) * dpsi * f;
        double day = delta * (std::cos(psi) * df - std::sin(psi) * dpsi * f);
        double amp = (ELECTRON_MASS * SPEED_OF_LIGHT_SQD * wavevector.t * d.a0) / ELEMENTARY_CHARGE;
        V3 E = (-amp) * V3(dax, day, 0.0);
        V3 B = (amp / SPEED_OF_LIGHT) * V3(day, -dax, 0.0);
        E = E.rotate_around_z(d.pol_angle);
        B = B.rotate_around_z(d.pol_angle);
        *E_out = E;
        *B_out = B;
        *a_out = ELEMENTARY_CHARGE * std::sqrt(E.norm_sqr()) / (ELECTRON_MASS * SPEED_OF_LIGHT * omega());
        return;
    }
    // FastFocusedLaser, fast_focused_laser.rs:190-218
    double phase = wavevector * r;
    double f, df;
    ffl_envelope(phase, &f, &df);
    V3 reE, imE, reB, imB;
    ffl_beam(r, &reE, &imE, &reB, &imB);
    V3 E = f * reE + df * imE;
    V3 B = f * reB + df * imB;
    if (d.polarization == PTG_POL_CIRCULAR) {
        V3 axis = wavevector.spatial().normalize();
        V3 rp = r.spatial().rotate_around(axis, -FRAC_PI_2);
        V4 r_prime(r.t, rp.x, rp.y, rp.z);
        ffl_beam(r_prime, &reE, &imE, &reB, &imB);
        V3 Ey = f * imE - df * reE;
        V3 By = f * imB - df * reB;
        E = E + Ey.rotate_around(axis, FRAC_PI_2);
        B = B + By.rotate_around(axis, FRAC_PI_2);
    }
    *E_out = E;
    *B_out = B;
    *a_out = ELEMENTARY_CHARGE * std::sqrt(E.norm_sqr()) / (ELECTRON_MASS * SPEED_OF_LIGHT * omega());
}

// focused_laser.rs:80-106
void Laser::fl_envelope(double phase, double* f, double* df) const {
    double nc = n_cycles();
    switch (d.envelope) {
        case PTG_ENV_COS2:
            if (std::fabs(phase) < PI * nc) {
                double env = powi(std::cos(phase / (2.0 * nc)), 4);
                *f = env;
                *df = 2.0 * wavevector.t * std::tan(phase / (2.0 * nc)) * env / nc;
            } else {
                *f = 0.0, *df = 0.0;
            }
            return;
        case PTG_ENV_FLATTOP:
            if (std::fabs(phase) > PI * (nc + 1.0)) {
                *f = 0.0, *df = 0.0;
            } else if (std::fabs(phase) > PI * (nc - 1.0)) {
                double arg = 0.25 * (std::fabs(phase) - (nc - 1.0) * PI);
                *f = powi(std::cos(arg), 4);
                *df = wavevector.t * signum(phase) * std::sin(arg) * powi(std::cos(arg), 3);
            } else {
                *f = 1.0, *df = 0.0;
            }
            return;
        default: {
            double tau = omega() * duration;
            double env = std::exp(-4.0 * LN_2 * powi(phase, 2) / powi(tau, 2));
            *f = env;
            *df = 8.0 * LN_2 * wavevector.t * phase * env / powi(tau, 2);
        }
    }
}

double Laser::a_sqd(const V4& r) const {
    double norm = d.polarization == PTG_POL_LINEAR ? 0.5 : 1.0;
    double phase = wavevector * r;
    if (d.model == PTG_PLANE_WAVE) {
        // plane_wave.rs:68-106
        double nc = d.n_cycles;
        switch (d.envelope) {
            case PTG_ENV_COS2:
                return std::fabs(phase) < PI * nc ? norm * powi(d.a0, 2) * powi(std::cos(phase / (2.0 * nc)), 4) : 0.0;
            case PTG_ENV_FLATTOP:
                if (std::fabs(phase) > PI * (nc + 1.0)) return 0.0;
                if (std::fabs(phase) > PI * (nc - 1.0)) {
                    double arg = 0.25 * (std::fabs(phase) - (nc - 1.0) * PI);
                    return norm * powi(d.a0, 2) * powi(std::cos(arg), 4);
                }
                return norm * powi(d.a0, 2);
            default: {
                double arg = -powi(phase / (PI * nc), 2);
                return norm * powi(d.a0, 2) * std::exp2(arg);
            }
        }
    }
    // focused_laser.rs:110-127
    double zr = 0.5 * wavevector.t * sq(d.waist);
    double width_sqd = 1.0 + powi(r.z / zr, 2);
    double rho_sqd = (powi(r.x, 2) + powi(r.y, 2)) / powi(d.waist, 2);
    double beam = norm * powi(d.a0, 2) * std::exp(-2.0 * rho_sqd / width_sqd) / width_sqd;
    double env, genv;
    fl_envelope(phase, &env, &genv);
    return beam * env;
}

V4 Laser::grad_a_sqd(const V4& r) const {
    double norm = d.polarization == PTG_POL_LINEAR ? 0.5 : 1.0;
    double phase = wavevector * r;
    if (d.model == PTG_PLANE_WAVE) {
        // plane_wave.rs:111-150
        double nc = d.n_cycles;
        double grad;
        switch (d.envelope) {
            case PTG_ENV_COS2:
                grad = std::fabs(phase) < PI * nc ? norm * wavevector.t * powi(d.a0, 2) * std::sin(phase / nc) *
                                                        powi(std::cos(phase / (2.0 * nc)), 2) / nc
                                                  : 0.0;
                break;
            case PTG_ENV_FLATTOP:
                if (std::fabs(phase) > PI * (nc + 1.0) || std::fabs(phase) < PI * (nc - 1.0)) {
                    grad = 0.0;
                } else {
                    double arg = 0.25 * (std::fabs(phase) - (nc - 1.0) * PI);
                    grad = norm * wavevector.t * powi(d.a0, 2) * signum(phase) * std::sin(arg) * powi(std::cos(arg), 3);
                }
                break;
            default: {
                double arg = -powi(phase / (PI * nc), 2);
                grad = norm * wavevector.t * powi(d.a0, 2) * 2.0 * LN_2 * phase * std::exp2(arg) / powi(PI * nc, 2);
            }
        }
        return V4(-grad, 0.0, 0.0, -grad);
    }
    // focused_laser.rs:131-161
    double zr = 0.5 * wavevector.t * sq(d.waist);
    double width_sqd = 1.0 + powi(r.z / zr, 2);
    double rho_sqd = (powi(r.x, 2) + powi(r.y, 2)) / powi(d.waist, 2);
    double beam = norm * powi(d.a0, 2) * std::exp(-2.0 * rho_sqd / width_sqd) / width_sqd;
    double gb0 = -4.0 * beam * r.x / (powi(d.waist, 2) * width_sqd);
    double gb1 = -4.0 * beam * r.y / (powi(d.waist, 2) * width_sqd);
    double gb2 = (2.0 * beam * r.z / (powi(zr, 2) * width_sqd)) * (2.0 * rho_sqd / width_sqd - 1.0);
    double env, genv;
    fl_envelope(phase, &env, &genv);
    double t = beam * genv + gb2 * env;
    return V4(-t, -(gb0 * env), -(gb1 * env), -t);
}

// lcf.rs:18-78
static void vay_push(const V4& r, const V4& ui, const V3& E, const V3& B, double rqm, double dt, int eqn, V4* r_out,
                     V4* u_out, double* dwork) {
    V3 u = ui.spatial();
    double gamma = std::sqrt(1.0 + u * u);
    V3 v = SPEED_OF_LIGHT * u / gamma;
    double alpha = rqm * dt / (2.0 * SPEED_OF_LIGHT);
    V3 u_half = u + alpha * (E + v.cross(B));
    double gamma_half = std::sqrt(1.0 + u_half * u_half);
    *dwork = rqm * (E * u_half) * dt / (gamma_half * SPEED_OF_LIGHT);
    V3 u_rad(0.0, 0.0, 0.0);
    if (eqn == LANDAU_LIFSHITZ || eqn == MODIFIED_LANDAU_LIFSHITZ) {
        double mag = std::sqrt(u_half.norm_sqr());
        V3 beta = u_half / mag;
        double E_rf_sqd = (E + SPEED_OF_LIGHT * beta.cross(B)).norm_sqr() - powi(E * beta, 2);
        double chi = E_rf_sqd > 0.0 ? gamma_half * std::sqrt(E_rf_sqd) / CRITICAL_FIELD : 0.0;
        double power = 2.0 * ALPHA_FINE * chi * chi / (3.0 * COMPTON_TIME);
        double g_chi = eqn == MODIFIED_LANDAU_LIFSHITZ ? gaunt_factor(chi) : 1.0;
        u_rad = g_chi * power * dt * u_half / mag;
    }
    V3 u_prime = u_half + alpha * E;
    double gamma_prime_sqd = 1.0 + u_prime * u_prime;
    V3 tau = alpha * SPEED_OF_LIGHT * B;
    double u_star = u_prime * tau;
    double sigma = gamma_prime_sqd - tau * tau;
    gamma = std::sqrt(0.5 * sigma + std::sqrt(0.25 * powi(sigma, 2) + tau * tau + powi(u_star, 2)));
    V3 t = tau / gamma;
    double s = 1.0 / (1.0 + t * t);
    V3 u_new = s * (u_prime + (u_prime * t) * t + u_prime.cross(t));
    u_new = u_new - u_rad;
    gamma = std::sqrt(1.0 + u_new * u_new);
    V4 un(gamma, u_new.x, u_new.y, u_new.z);
    *u_out = un;
    *r_out = r + 0.5 * SPEED_OF_LIGHT * un * dt / gamma;
}

void Laser::push(const V4& r0, const V4& u0, double rqm, double dt, int eqn, V4* r_out, V4* u_out, double* dt_out,
                 double* dwork) const {
    if (lcfa()) {
        // field/mod.rs:147-152
        V4 r = r0 + 0.5 * SPEED_OF_LIGHT * u0 * dt / u0.t;
        V3 E, B;
        double a;
        fields(r, &E, &B, &a);
        vay_push(r, u0, E, B, rqm, dt, eqn, r_out, u_out, dwork);
        *dt_out = dt;
        return;
    }
    // plane_wave.rs:196-249 == focused_laser.rs:205-258 (modified LL is
    // rejected at option parsing for LMA, main.rs:373-380)
    double dtau = dt / u0.t;
    double scale = powi(rqm / (ELECTRON_CHARGE / ELECTRON_MASS), 2);
    V4 u_mid(0, 0, 0, 0);
    auto ll_force = [&](const V4& rr, const V4& uu) {
        double eta = SPEED_OF_LIGHT * COMPTON_TIME * (wavevector * uu);
        return (-2.0 * ALPHA_FINE * a_sqd(rr) * powi(eta, 2)) * uu / (3.0 * COMPTON_TIME);
    };
    auto ll_work = [&](const V4& rr, const V4& uu) {
        double eta = SPEED_OF_LIGHT * COMPTON_TIME * (wavevector * uu);
        double om = SPEED_OF_LIGHT * wavevector.t;
        double delta = d.polarization == PTG_POL_CIRCULAR ? 1.0 : 0.75;
        return 2.0 * ALPHA_FINE * om * eta * delta * powi(a_sqd(rr), 2) / 3.0;
    };
    bool rr = eqn == LANDAU_LIFSHITZ;
    if (rr) {
        V4 f = (0.5 * SPEED_OF_LIGHT * scale) * grad_a_sqd(r0);
        V4 g = powi(scale, 2) * ll_force(r0, u0);
        u_mid = u0 + 0.5 * (f + g) * dtau;
    }
    V4 r = r0 + 0.5 * SPEED_OF_LIGHT * u0 * dtau;
    double dt_actual = 0.5 * u0.t * dtau;
    V4 f = (0.5 * SPEED_OF_LIGHT * scale) * grad_a_sqd(r);
    V4 g = rr ? powi(scale, 2) * ll_force(r, u_mid) : V4(0, 0, 0, 0);
    V4 u = u0 + (f + g) * dtau;
    *dwork = rr ? (f.t + ll_work(r, u_mid)) * dtau : f.t * dtau;
    r = r + 0.5 * SPEED_OF_LIGHT * u * dtau;
    dt_actual = dt_actual + 0.5 * u.t * dtau;
    double b = 1.0 + a_sqd(r);
    u = V4(std::sqrt(b + u.x * u.x + u.y * u.y + u.z * u.z), u.x, u.y, u.z);
    *r_out = r;
    *u_out = u;
    *dt_out = dt_actual;
}

int Laser::radiate(const V4& r, const V4& u, double dt, DrawStream& rng, bool classical, bool* emitted,
                   RadiationEvent* ev, uint64_t* rejections) const {
    *emitted = false;
    if (!lcfa()) return lma_radiate(*this, r, u, dt, rng, classical, emitted, ev, rejections);
    // lcf.rs:85-134
    V3 E, B;
    double a;
    fields(r, &E, &B, &a);
    V3 beta = u.spatial() / u.t;
    double E_rf_sqd = (E + SPEED_OF_LIGHT * beta.cross(B)).norm_sqr() - powi(E * beta, 2);
    double chi = E_rf_sqd > 0.0 ? u.t * std::sqrt(E_rf_sqd) / CRITICAL_FIELD : 0.0;
    double prob = classical ? dt * lcfa_classical_rate(chi, u.t) : dt * lcfa_photon_rate(chi, u.t);
    if (rng.next() < prob) {
        double r1 = rng.next(), r2 = rng.next(), r3 = rng.next();
        double omega_mc2, theta, cphi;
        bool has_theta;
        if (classical)
            lcfa_classical_sample(chi, u.t, r1, r2, r3, &omega_mc2, &has_theta, &theta, &cphi);
        else
            lcfa_photon_sample(chi, u.t, r1, r2, r3, &omega_mc2, &has_theta, &theta, &cphi);
        if (has_theta) {
            V3 lng = beta.normalize();
            V3 w = -(E - (lng * E) * lng / std::sqrt(E.norm_sqr()) + SPEED_OF_LIGHT * beta.cross(B)).normalize();
            V3 perp = w.rotate_around(lng, cphi);
            V3 k3 = omega_mc2 * (std::cos(theta) * lng + std::sin(theta) * perp);
            V4 k = V4::lightlike(k3.x, k3.y, k3.z);
            Stokes pol = classical ? lcfa_classical_stokes_parameters(k, chi, u.t, beta, w)
                                   : lcfa_stokes_parameters(k, chi, u.t, beta, w);
            ev->k = k;
            ev->u_prime = u - k;
            ev->pol = pol;
            ev->a_eff = a;
            ev->chi = chi;
            ev->absorption = 0.0;
            *emitted = true;
        }
    }
    return PTG_OK;
}

int Laser::pair_create(const V4& r, const V4& ell, const Stokes& sv, double dt, DrawStream& rng, double rate_increase,
                       double* prob_out, Stokes* sv_new, bool* created, PairEvent* ev, uint64_t* rejections) const {
    *created = false;
    if (!lcfa())
        return lma_pair_create(*this, r, ell, sv, dt, rng, rate_increase, prob_out, sv_new, created, ev, rejections);
    // lcf.rs:144-193
    V3 E, B;
    double a;
    fields(r, &E, &B, &a);
    V3 n = ell.spatial().normalize();
    V3 a_perp = E - (E * n) * n + SPEED_OF_LIGHT * n.cross(B);
    double E_rf_sqd = a_perp.norm_sqr();
    double chi = 0.0, prob = 0.0;
    Stokes svn = sv;
    if (E_rf_sqd > 0.0) {
        chi = ell.t * std::sqrt(E_rf_sqd) / CRITICAL_FIELD;
        prob = lcfa_pair_probability(ell, sv, chi, a_perp, dt, &svn);
    }
    *prob_out = prob;
    *sv_new = svn;
    double ri = (prob * rate_increase > 0.1) ? 0.1 / prob : rate_increase;
    if (rng.next() < prob * ri) {
        double gamma_p, cos_theta, cphi, s, z;
        if (!lcfa_pair_sample(ell, sv, chi, a_perp, rng, &gamma_p, &cos_theta, &cphi, &s, &z))
            return PTG_ERR_REJECTION_CAP;
        double sin_theta = std::sqrt(1.0 - cos_theta * cos_theta);
        double up = gamma_p * std::sqrt(1.0 - 1.0 / (gamma_p * gamma_p));
        V3 e1 = a_perp.normalize();
        V3 e2 = n.cross(e1);
        V3 u_p = up * (cos_theta * n + sin_theta * std::cos(cphi) * e1 + sin_theta * std::sin(cphi) * e2);
        V3 u_e = ell.spatial() - u_p;
        ev->u_p = V4(0.0, u_p.x, u_p.y, u_p.z).unitize();
        ev->u_e = V4(0.0, u_e.x, u_e.y, u_e.z).unitize();
        ev->frac = 1.0 / ri;
        ev->a_eff = a;
        ev->chi = chi;
        ev->absorption = 0.0;
        *created = true;
    }
    return PTG_OK;
}

// ------------------------------------------------------------ collide ---
static double rqm_of(int species) {
    if (species == PTG_ELECTRON) return ELECTRON_CHARGE / ELECTRON_MASS;
    if (species == PTG_POSITRON) return -ELECTRON_CHARGE / ELECTRON_MASS;
    return 0.0;
}

// main.rs:134-289
// A bound on any one particle's steps, so that a run of the oracle always
// ends: the reference steps a particle until it leaves the field, which a
// photon moving almost with the laser (its phase k(t - z) advancing by ever
// less) may take without limit to do.  A particle at the bound is retired
// with PTG_ERR_REJECTION_CAP, as the device's own step cap does.
constexpr uint32_t ORACLE_STEP_CAP = 1u << 26;

void collide(const Laser& laser, const ptg_collide_options& o, const OracleParticle& incident, uint64_t seed,
             uint64_t* current_id, std::vector<OracleParticle>& out, OracleStats& st) {
    std::vector<OracleParticle> stack;
    stack.push_back(incident);
    std::vector<OracleParticle> secondaries, intermediates;
    double dt = laser.max_timestep() * o.dt_multiplier;
    uint64_t primary_id = incident.id;
    int eqn = LORENTZ;
    if (o.classical && o.rr) eqn = o.gaunt_factor ? MODIFIED_LANDAU_LIFSHITZ : LANDAU_LIFSHITZ;
    bool classical_mode = o.classical && !o.gaunt_factor;
    bool electron_recoils = !o.classical && o.rr;
    double t_stop = o.t_stop;

    while (!stack.empty()) {
        OracleParticle pt = stack.back();
        stack.pop_back();
        bool untracked = (!o.tracking_secondaries && pt.id != primary_id) ||
                         (o.max_generation >= 0 && pt.generation > o.max_generation);
        if (untracked) {
            secondaries.push_back(pt);
            continue;
        }
        DrawStream rng;
        rng.seed = seed;
        rng.stream = pt.stream;
        uint32_t step = 0;
        if (pt.species != PTG_PHOTON) {
            double rqm = rqm_of(pt.species);
            while (laser.contains(pt.r) && pt.r.t / SPEED_OF_LIGHT < t_stop) {
                if (step >= ORACLE_STEP_CAP) {
                    pt.status = PTG_ERR_REJECTION_CAP;
                    break;
                }
                rng.begin_step(step);
                V4 r, u;
                double dt_actual, work;
                laser.push(pt.r, pt.u, rqm, dt, eqn, &r, &u, &dt_actual, &work);
                bool emitted;
                RadiationEvent ev;
                int err = laser.radiate(r, u, dt_actual, rng, classical_mode, &emitted, &ev, &st.rejections);
                st.lepton_steps++;
                if (err != PTG_OK) {
                    pt.status = err;
                    pt.r = r;
                    pt.u = u;
                    break;
                }
                if (emitted) {
                    OracleParticle ph{};
                    ph.species = PTG_PHOTON;
                    ph.r = r;
                    ph.r0 = r;
                    ph.u = ev.k;
                    ph.u0 = V4(0, 0, 0, 0);
                    ph.pol = ev.pol;
                    ph.weight = pt.weight;
                    ph.payload = ev.a_eff;
                    ph.parent_chi = ev.chi;
                    ph.id = (*current_id)++;
                    ph.parent_id = pt.id;
                    ph.primary = pt.primary;
                    ph.stream = child_stream(pt.stream, step, 0);
                    ph.generation = pt.generation + 1;
                    stack.push_back(ph);
                    st.emissions++;
                    st.created++;
                    if (electron_recoils) u = ev.u_prime;
                    pt.interaction_count += 1.0;
                    if (!o.classical) pt.work += ev.absorption;
                }
                pt.r = r;
                pt.u = u;
                pt.work += work;
                ++step;
            }
            if (pt.id != primary_id || !o.discard_bg_e || pt.interaction_count > 0.0) secondaries.push_back(pt);
        } else {
            bool decayed = false;
            while (laser.contains(pt.r) && pt.r.t / SPEED_OF_LIGHT < t_stop && !decayed && o.tracking_photons) {
                if (step >= ORACLE_STEP_CAP) {
                    pt.status = PTG_ERR_REJECTION_CAP;
                    break;
                }
                rng.begin_step(step);
                V4 ell = pt.u;
                V4 r = pt.r + SPEED_OF_LIGHT * ell * dt / ell.t;
                Stokes pol = o.pol_resolved ? pt.pol : Stokes::unpolarized();
                double prob;
                Stokes pol_new;
                bool created;
                PairEvent ev;
                int err = laser.pair_create(r, ell, pol, dt, rng, o.rate_increase, &prob, &pol_new, &created, &ev,
                                            &st.rejections);
                st.photon_steps++;
                if (err != PTG_OK) {
                    pt.status = err;
                    pt.r = r;
                    break;
                }
                if (created) {
                    uint64_t id = *current_id;
                    *current_id += 2;
                    for (int k = 0; k < 2; ++k) {
                        OracleParticle lp{};
                        lp.species = k == 0 ? PTG_ELECTRON : PTG_POSITRON;
                        lp.r = r;
                        lp.r0 = r;
                        lp.u = k == 0 ? ev.u_e : ev.u_p;
                        lp.u0 = V4(1, 0, 0, 0);
                        lp.pol = Stokes::unpolarized();
                        lp.weight = ev.frac * pt.weight;
                        lp.payload = ev.a_eff;
                        lp.parent_chi = ev.chi;
                        lp.work = 0.5 * ev.absorption;
                        lp.id = id + k;
                        lp.parent_id = pt.id;
                        lp.primary = pt.primary;
                        lp.stream = child_stream(pt.stream, step, 1 + k);
                        lp.generation = pt.generation + 1;
                        stack.push_back(lp);
                    }
                    st.pair_events++;
                    st.created += 2;
                    if (ev.frac == 1.0)
                        decayed = true;
                    else
                        pt.weight = pt.weight * (1.0 - ev.frac);
                }
                if (o.rotate_stokes_pars && o.pol_resolved) pt.pol = pol_new;
                pt.interaction_count += prob;
                pt.r = r;
                ++step;
            }
            if (!decayed && (pt.id != primary_id || !o.discard_bg_ph)) secondaries.push_back(pt);
            if (decayed && o.keep_decayed_photons) {
                pt.flags |= 1;
                intermediates.push_back(pt);
            }
        }
    }

    // main.rs:271-282
    V3 n0 = (ELECTRON_MASS_MEV * incident.u).spatial().normalize();
    std::vector<OracleParticle> kept;
    double cmax = std::cos(o.max_angle);
    for (auto& pt : secondaries) {
        V4 p = ELECTRON_MASS_MEV * pt.u;
        V3 n = p.spatial().normalize();
        if (pt.status != PTG_OK || (p.t > o.min_energy && n0 * n > cmax)) kept.push_back(pt);
    }
    if (o.multiplicity >= 0 && kept.size() != (size_t)o.multiplicity + 1) kept.clear();
    for (auto& pt : kept) out.push_back(pt);
    for (auto& pt : intermediates) out.push_back(pt);
}

}  // namespace orc
