// The four field models of ptarmigan on the device: FastPlaneWave and
// FastFocusedLaser (explicit E, B; LCFA) and PlaneWave and FocusedLaser
// (cycle-averaged <a^2>; LMA), plus the particle pushers.
#pragma once
#include "ptg_math.cuh"

namespace ptg {

enum { M_PLANE_WAVE = 0, M_FAST_PLANE_WAVE = 1, M_FOCUSED_LASER = 2, M_FAST_FOCUSED_LASER = 3 };
enum { ENV_COS2 = 0, ENV_FLATTOP = 1, ENV_GAUSSIAN = 2 };
enum { EQN_LORENTZ = 0, EQN_LL = 1, EQN_MODIFIED_LL = 2 };

// Laser constants derived once on the host from ptg_laser_desc.
struct FieldParams {
    int model, circular, envelope, finite_bandwidth;
    double a0, k;              // wavenumber 2 pi / lambda; wavevector = k (1, 0, 0, 1)
    double omega;              // c k
    double n_cycles;           // for focused models: c * duration * k / (2 pi)
    double duration;
    double waist, zr, eps;     // waist, Rayleigh range, waist / zr
    double pol_angle, cos_pa, sin_pa;
    double chirp_b;
    double E0, B0;             // focused LCFA amplitude
    double amp;                // plane-wave LCFA amplitude m c^2 k a0 / e
    double max_phase;          // Field::contains
    double bandwidth;          // LMA finite-bandwidth width
    double env_cut;            // |phase| beyond which the envelope is below 1e-18: E = B = 0 (0 = off)
    double inv_waist, inv_zr;  // reciprocals, so the per-step field needs no division
    double inv_tau;            // 1 / (omega * duration)
    double chi_scale;          // field scale of lcfa_fields32 over the critical field
    double drift_ell_max;      // LCFA photons with ell^0 below this never create pairs (0 = off)
    double lma_cut;            // LMA: |phase| beyond which <a^2> < 2^-60 (0 = off)
    double inv_w2, asq0, env_c; // focused LMA: 1 / waist^2, norm a0^2, 4 ln 2 / (omega duration)^2
    // FP32 copies for the per-step FP32 path (converted once on the host,
    // the same rounding as a conversion on the device)
    float eps32, cos_pa32, sin_pa32, inv_tau32, chi_scale32;
};

__device__ __forceinline__ double phase_of(const FieldParams& f, d4 r) { return f.k * r.t - f.k * r.z; }

__device__ __forceinline__ bool contains(const FieldParams& f, d4 r) { return phase_of(f, r) < f.max_phase; }

// ---------------------------------------------- FastPlaneWave (LCFA) -----
// fast_plane_wave.rs:121-195 (no compensating-chirp feature)
__device__ __forceinline__ void fpw_fields(const FieldParams& f, d4 r, d3* E, d3* B, double* a) {
    double delta = f.circular ? 1.0 : 0.0;
    double phi = phase_of(f, r);
    double psi = phi * (1.0 + f.chirp_b * phi);
    double dpsi = 1.0 + 2.0 * f.chirp_b * phi;
    double nc = f.n_cycles;
    double env, denv;
    if (f.envelope == ENV_COS2) {
        if (fabs(phi) < nc * PI) {
            double c = cos(phi / (2.0 * nc));
            env = c * c;
            denv = -sin(phi / nc) / (2.0 * nc);
        } else {
            env = 0.0, denv = 0.0;
        }
    } else if (f.envelope == ENV_FLATTOP) {
        if (fabs(phi) > PI * (nc + 1.0)) {
            env = 0.0, denv = 0.0;
        } else if (fabs(phi) > PI * (nc - 1.0)) {
            double arg = 0.25 * (fabs(phi) - (nc - 1.0) * PI);
            double c = cos(arg);
            env = c * c;
            denv = -dsign(phi) * 0.25 * sin(2.0 * arg);
        } else {
            env = 1.0, denv = 0.0;
        }
    } else {
        double q = phi / (PI * nc);
        double e2 = exp2(-0.5 * (q * q));
        env = e2;
        denv = -LN_2 * phi * e2 / ((PI * nc) * (PI * nc));
    }
    double sp, cp;
    sincos(psi, &sp, &cp);
    double dax = sp * denv + cp * dpsi * env;
    double day = delta * (cp * denv - sp * dpsi * env);
    d3 e = mk3(-f.amp * dax, -f.amp * day, -f.amp * 0.0);
    double bs = f.amp / SPEED_OF_LIGHT;
    d3 b = mk3(bs * day, bs * (-dax), 0.0);
    *E = mk3(f.cos_pa * e.x - f.sin_pa * e.y, f.cos_pa * e.y + f.sin_pa * e.x, e.z);
    *B = mk3(f.cos_pa * b.x - f.sin_pa * b.y, f.cos_pa * b.y + f.sin_pa * b.x, b.z);
    *a = ELEMENTARY_CHARGE * sqrt(norm_sqr(*E)) / (ELECTRON_MASS * SPEED_OF_LIGHT * f.omega);
}

// ------------------------------------------- FastFocusedLaser (LCFA) -----
struct cplx {
    double re, im;
};
__device__ __forceinline__ cplx cmul(cplx a, cplx b) { return cplx{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ __forceinline__ cplx cadd(cplx a, cplx b) { return cplx{a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ cplx cscale(double s, cplx a) { return cplx{s * a.re, s * a.im}; }
__device__ __forceinline__ cplx cadds(double s, cplx a) { return cplx{s + a.re, a.im}; }
__device__ __forceinline__ cplx cmul_i(cplx a) { return cplx{-a.im, a.re}; }
__device__ __forceinline__ cplx cmul_mi(cplx a) { return cplx{a.im, -a.re}; }

// Salamin's O(eps^4) Gaussian-beam fields (fast_focused_laser.rs:59-111),
// for the beam polarised along x after undoing pol_angle.  The carrier
// phase is k.r.  Returns Re/Im parts of E and B, already scaled by E0/B0
// and rotated back by pol_angle (rotation supplied as (cr, sr)).
//
// Precision split: the terms of order eps^0 and eps^1 (the paraxial beam
// and the first longitudinal components) are FP64; the diffraction
// corrections of order eps^2..eps^4, whose size relative to the leading
// term is at most ~eps^2 rho^4 (eps = w0 / zR, 0.06 for w0 = 4 um), are
// evaluated in FP32 and applied in FP64.  Their rounding (~6e-8 of a term
// that is itself <= ~1e-2 of the field where the beam is not negligible)
// puts the field error near 1e-9 of E0.
__device__ __forceinline__ void ffl_beam(const FieldParams& f, d4 r, double cr, double sr, d3* reE, d3* imE, d3* reB,
                                         d3* imB) {
    // r.rotate_around_z(-angle)
    double rx = cr * r.x + sr * r.y;
    double ry = cr * r.y - sr * r.x;
    double x = rx * f.inv_waist, y = ry * f.inv_waist, z = r.z * f.inv_zr;
    double rho2 = x * x + y * y;
    // f = i / (z + i) = (1 + i z) / (1 + z^2)
    double den = 1.0 / (1.0 + z * z);
    double fre = den, fim = z * den;
    // prefactor = f exp(-f rho^2 + i phase)
    double ph = f.k * r.t - f.k * r.z;
    double ex = exp(-fre * rho2);
    double sn, cs;
    sincos(ph - fim * rho2, &sn, &cs);
    cplx pre = cmul(cplx{fre, fim}, cplx{ex * cs, ex * sn});
    // corrections in FP32
    float xf = (float)x, yf = (float)y, r2 = (float)rho2;
    float ef = f.eps32, e2 = ef * ef, e3 = e2 * ef, e4 = e2 * e2;
    float fr = (float)fre, fi = (float)fim;
    float f2r = fr * fr - fi * fi, f2i = 2.0f * fr * fi;
    float f3r = f2r * fr - f2i * fi, f3i = f2r * fi + f2i * fr;
    float f4r = f2r * f2r - f2i * f2i, f4i = 2.0f * f2r * f2i;
    float r4 = r2 * r2, r6 = r4 * r2, r8 = r4 * r4;
    auto mul = [](float ar, float ai, float br, float bi, float* cr_, float* ci_) {
        *cr_ = ar * br - ai * bi;
        *ci_ = ar * bi + ai * br;
    };
    float tr, ti, ur, ui;
    // Ex: eps^2 f^2 (x^2 - f rho^4/4) + eps^4 f^2 (1/8 - f rho^2/4 + f^2 (x^2 rho^2 - rho^4/16)
    //     + f^3 rho^4 (-x^2 - rho^2/2)/4 + f^4 rho^8/32)
    float t2r = xf * xf - 0.25f * r4 * fr, t2i = -0.25f * r4 * fi;
    float t4r = 0.125f - 0.25f * r2 * fr + (xf * xf * r2 - 0.0625f * r4) * f2r + 0.25f * r4 * (-xf * xf - 0.5f * r2) * f3r +
                0.03125f * r8 * f4r;
    float t4i = -0.25f * r2 * fi + (xf * xf * r2 - 0.0625f * r4) * f2i + 0.25f * r4 * (-xf * xf - 0.5f * r2) * f3i +
                0.03125f * r8 * f4i;
    mul(f2r, f2i, e2 * t2r + e4 * t4r, e2 * t2i + e4 * t4i, &tr, &ti);
    cplx cX = cplx{(double)tr, (double)ti};
    // Ey: eps^2 f^2 x y + eps^4 x y f^4 rho^2 (1 - f rho^2/4)
    mul(f4r, f4i, 1.0f - 0.25f * r2 * fr, -0.25f * r2 * fi, &ur, &ui);
    cplx cY = cplx{(double)(e2 * xf * yf * f2r + e4 * xf * yf * r2 * ur), (double)(e2 * xf * yf * f2i + e4 * xf * yf * r2 * ui)};
    // Ez: eps f x (FP64) + eps^3 f^2 x (-1/2 + f rho^2 - f^2 rho^4/4)
    mul(f2r, f2i, -0.5f + r2 * fr - 0.25f * r4 * f2r, r2 * fi - 0.25f * r4 * f2i, &tr, &ti);
    cplx cZ = cplx{f.eps * x * fre + (double)(e3 * xf * tr), f.eps * x * fim + (double)(e3 * xf * ti)};
    // By: eps^2 f^2 rho^2 (1 - f rho^2/2)/2 + eps^4 f^2 (-1 + 2 f rho^2 + 2.5 f^2 rho^4 - 2 f^3 rho^6 + f^4 rho^8/4)/8
    float b2r = 0.5f * r2 * (1.0f - 0.5f * r2 * fr), b2i = 0.5f * r2 * (-0.5f * r2 * fi);
    float b4r = -1.0f + 2.0f * r2 * fr + 2.5f * r4 * f2r - 2.0f * r6 * f3r + 0.25f * r8 * f4r;
    float b4i = 2.0f * r2 * fi + 2.5f * r4 * f2i - 2.0f * r6 * f3i + 0.25f * r8 * f4i;
    mul(f2r, f2i, e2 * b2r + 0.125f * e4 * b4r, e2 * b2i + 0.125f * e4 * b4i, &tr, &ti);
    cplx cB = cplx{(double)tr, (double)ti};
    // Bz: eps f y (FP64) + eps^3 f^2 y (1 + f rho^2 - f^2 rho^4/2)/2
    mul(f2r, f2i, 0.5f * (1.0f + r2 * fr - 0.5f * r4 * f2r), 0.5f * (r2 * fi - 0.5f * r4 * f2i), &tr, &ti);
    cplx cBz = cplx{f.eps * y * fre + (double)(e3 * yf * tr), f.eps * y * fim + (double)(e3 * yf * ti)};
    cplx Ex = cmul_mi(cmul(pre, cadds(1.0, cX)));
    cplx Ey = cmul_mi(cmul(pre, cY));
    cplx Ez = cmul(pre, cZ);
    cplx By = cmul_mi(cmul(pre, cadds(1.0, cB)));
    cplx Bz = cmul(pre, cBz);
    // scale and rotate by +angle
    double E0 = f.E0, B0 = f.B0;
    *reE = mk3(E0 * (cr * Ex.re - sr * Ey.re), E0 * (cr * Ey.re + sr * Ex.re), E0 * Ez.re);
    *imE = mk3(E0 * (cr * Ex.im - sr * Ey.im), E0 * (cr * Ey.im + sr * Ex.im), E0 * Ez.im);
    *reB = mk3(B0 * (-sr * By.re), B0 * (cr * By.re), B0 * Bz.re);
    *imB = mk3(B0 * (-sr * By.im), B0 * (cr * By.im), B0 * Bz.im);
}

// fast_focused_laser.rs:123-151
__device__ __forceinline__ void ffl_envelope(const FieldParams& f, double phase, double* env, double* denv) {
    double nc = f.n_cycles;
    if (f.envelope == ENV_COS2) {
        if (fabs(phase) < PI * nc) {
            double c = cos(phase / (2.0 * nc));
            double e = c * c;
            *env = e;
            *denv = -1.0 * tan(phase / (2.0 * nc)) * e / nc;
        } else {
            *env = 0.0, *denv = 0.0;
        }
    } else if (f.envelope == ENV_FLATTOP) {
        if (fabs(phase) > PI * (nc + 1.0)) {
            *env = 0.0, *denv = 0.0;
        } else if (fabs(phase) > PI * (nc - 1.0)) {
            double arg = 0.25 * (fabs(phase) - (nc - 1.0) * PI);
            double c = cos(arg);
            *env = c * c;
            *denv = -0.25 * dsign(phase) * sin(2.0 * arg);
        } else {
            *env = 1.0, *denv = 0.0;
        }
    } else {
        double q = phase * f.inv_tau;
        double e = exp(-2.0 * LN_2 * (q * q));
        *env = e;
        *denv = -4.0 * LN_2 * q * f.inv_tau * e;
    }
}

// fast_focused_laser.rs:190-218
__device__ __forceinline__ void ffl_fields(const FieldParams& f, d4 r, d3* E, d3* B, double* a) {
    double phase = phase_of(f, r);
    if (f.env_cut > 0.0 && fabs(phase) > f.env_cut) {
        // envelope below 1e-300: the fields are zero to every bit that can
        // reach u (and the reference's own values underflow to 0 soon after)
        *E = mk3(0.0, 0.0, 0.0);
        *B = mk3(0.0, 0.0, 0.0);
        *a = 0.0;
        return;
    }
    double env, denv;
    ffl_envelope(f, phase, &env, &denv);
    d3 reE, imE, reB, imB;
    ffl_beam(f, r, f.cos_pa, f.sin_pa, &reE, &imE, &reB, &imB);
    d3 e = env * reE + denv * imE;
    d3 b = env * reB + denv * imB;
    if (f.circular) {
        // second beam: r rotated by -pi/2 about z, fields rotated by +pi/2
        d4 rp = d4{r.t, r.y, -r.x, r.z};
        ffl_beam(f, rp, 1.0, 0.0, &reE, &imE, &reB, &imB);
        d3 ey = env * imE - denv * reE;
        d3 by = env * imB - denv * reB;
        e = e + mk3(-ey.y, ey.x, ey.z);
        b = b + mk3(-by.y, by.x, by.z);
    }
    *E = e;
    *B = b;
    *a = ELEMENTARY_CHARGE * sqrt(norm_sqr(e)) / (ELECTRON_MASS * SPEED_OF_LIGHT * f.omega);
}

__device__ __forceinline__ void lcfa_fields(const FieldParams& f, d4 r, d3* E, d3* B, double* a) {
    if (f.model == M_FAST_PLANE_WAVE)
        fpw_fields(f, r, E, B, a);
    else
        ffl_fields(f, r, E, B, a);
}

// ------------------------------------------------------- LCF push -------
// lcf.rs:18-78 (Vay pusher with optional classical radiation reaction).
// gaunt: g(chi) for the modified LL equation (computed by the caller's
// functor, 1 otherwise).
template <typename Gaunt>
__device__ __forceinline__ void vay_push(d4 r, d4 ui, d3 E, d3 B, double rqm, double dt, int eqn, Gaunt gaunt,
                                         d4* r_out, d4* u_out, double* dwork, double* h_out = nullptr) {
    // the same algebra as the reference; where only 1 / gamma is needed it
    // comes from one reciprocal square root instead of a square root and a
    // division (each about ten FP64 instructions here), which moves results
    // by an ulp or two
    d3 u = mk3(ui.x, ui.y, ui.z);
    double ig = rsqrt(1.0 + dot(u, u));  // 1 / gamma
    d3 v = (SPEED_OF_LIGHT * ig) * u;
    double alpha = rqm * dt * (0.5 / SPEED_OF_LIGHT);
    d3 u_half = u + alpha * (E + cross(v, B));
    double g2_half = 1.0 + dot(u_half, u_half);
    *dwork = (2.0 * alpha) * dot(E, u_half) * rsqrt(g2_half);
    d3 u_rad = mk3(0.0, 0.0, 0.0);
    if (eqn != EQN_LORENTZ) {
        double gamma_half = sqrt(g2_half);
        double mag = sqrt(norm_sqr(u_half));
        double imag = 1.0 / mag;
        d3 beta = imag * u_half;
        double eb = dot(E, beta);
        double E_rf_sqd = norm_sqr(E + SPEED_OF_LIGHT * cross(beta, B)) - eb * eb;
        double chi = E_rf_sqd > 0.0 ? gamma_half * sqrt(E_rf_sqd) / CRITICAL_FIELD : 0.0;
        double power = 2.0 * ALPHA_FINE * chi * chi / (3.0 * COMPTON_TIME);
        double g = eqn == EQN_MODIFIED_LL ? gaunt(chi) : 1.0;
        u_rad = (g * power * dt * imag) * u_half;
    }
    d3 up = u_half + alpha * E;
    double gp2 = 1.0 + dot(up, up);
    d3 tau = (alpha * SPEED_OF_LIGHT) * B;
    double ustar = dot(up, tau);
    double sigma = gp2 - dot(tau, tau);
    double ig_new = rsqrt(0.5 * sigma + sqrt(0.25 * (sigma * sigma) + dot(tau, tau) + ustar * ustar));
    d3 t = ig_new * tau;
    double s = 1.0 / (1.0 + dot(t, t));
    d3 un = s * (up + dot(up, t) * t + cross(up, t));
    un = un - u_rad;
    double g2 = 1.0 + dot(un, un);
    double ign = rsqrt(g2);
    double gamma = g2 * ign;  // sqrt(g2) to an ulp or two
    d4 u4 = d4{gamma, un.x, un.y, un.z};
    double h = (0.5 * SPEED_OF_LIGHT * dt) * ign;
    *u_out = u4;
    *r_out = d4{r.t + h * u4.t, r.x + h * u4.x, r.y + h * u4.y, r.z + h * u4.z};
    if (h_out) *h_out = h;  // also the next step's first half-drift factor
}

// ---------------------------------------------------- LMA envelopes ------
// plane_wave.rs:68-150 and focused_laser.rs:80-161: <a^2>(r) and its
// raised four-gradient.
__device__ __forceinline__ double lma_a_sqd(const FieldParams& f, d4 r) {
    double norm = f.circular ? 1.0 : 0.5;
    double phase = phase_of(f, r);
    double nc = f.n_cycles;
    double a02 = f.a0 * f.a0;
    if (f.model == M_PLANE_WAVE) {
        if (f.envelope == ENV_COS2) {
            if (fabs(phase) < PI * nc) {
                double c = cos(phase / (2.0 * nc));
                return norm * a02 * powi(c, 4);
            }
            return 0.0;
        } else if (f.envelope == ENV_FLATTOP) {
            if (fabs(phase) > PI * (nc + 1.0)) return 0.0;
            if (fabs(phase) > PI * (nc - 1.0)) {
                double arg = 0.25 * (fabs(phase) - (nc - 1.0) * PI);
                return norm * a02 * powi(cos(arg), 4);
            }
            return norm * a02;
        }
        double q = phase / (PI * nc);
        return norm * a02 * exp2(-(q * q));
    }
    double wsq = 1.0 + (r.z / f.zr) * (r.z / f.zr);
    double rho2 = (r.x * r.x + r.y * r.y) / (f.waist * f.waist);
    double beam = norm * a02 * exp(-2.0 * rho2 / wsq) / wsq;
    double env;
    if (f.envelope == ENV_COS2) {
        env = fabs(phase) < PI * nc ? powi(cos(phase / (2.0 * nc)), 4) : 0.0;
    } else if (f.envelope == ENV_FLATTOP) {
        if (fabs(phase) > PI * (nc + 1.0))
            env = 0.0;
        else if (fabs(phase) > PI * (nc - 1.0))
            env = powi(cos(0.25 * (fabs(phase) - (nc - 1.0) * PI)), 4);
        else
            env = 1.0;
    } else {
        double tau = f.omega * f.duration;
        env = exp(-4.0 * LN_2 * phase * phase / (tau * tau));
    }
    return beam * env;
}

__device__ __forceinline__ d4 lma_grad_a_sqd(const FieldParams& f, d4 r) {
    double norm = f.circular ? 1.0 : 0.5;
    double phase = phase_of(f, r);
    double nc = f.n_cycles;
    double a02 = f.a0 * f.a0;
    double kk = f.k;
    if (f.model == M_PLANE_WAVE) {
        double grad;
        if (f.envelope == ENV_COS2) {
            if (fabs(phase) < PI * nc) {
                double c = cos(phase / (2.0 * nc));
                grad = norm * kk * a02 * sin(phase / nc) * (c * c) / nc;
            } else {
                grad = 0.0;
            }
        } else if (f.envelope == ENV_FLATTOP) {
            if (fabs(phase) > PI * (nc + 1.0) || fabs(phase) < PI * (nc - 1.0)) {
                grad = 0.0;
            } else {
                double arg = 0.25 * (fabs(phase) - (nc - 1.0) * PI);
                grad = norm * kk * a02 * dsign(phase) * sin(arg) * powi(cos(arg), 3);
            }
        } else {
            double q = phase / (PI * nc);
            grad = norm * kk * a02 * 2.0 * LN_2 * phase * exp2(-(q * q)) / ((PI * nc) * (PI * nc));
        }
        return d4{-grad, 0.0, 0.0, -grad};
    }
    double wsq = 1.0 + (r.z / f.zr) * (r.z / f.zr);
    double w2 = f.waist * f.waist;
    double rho2 = (r.x * r.x + r.y * r.y) / w2;
    double beam = norm * a02 * exp(-2.0 * rho2 / wsq) / wsq;
    double gb0 = -4.0 * beam * r.x / (w2 * wsq);
    double gb1 = -4.0 * beam * r.y / (w2 * wsq);
    double gb2 = (2.0 * beam * r.z / (f.zr * f.zr * wsq)) * (2.0 * rho2 / wsq - 1.0);
    double env, genv;
    if (f.envelope == ENV_COS2) {
        if (fabs(phase) < PI * nc) {
            double e = powi(cos(phase / (2.0 * nc)), 4);
            env = e;
            genv = 2.0 * kk * tan(phase / (2.0 * nc)) * e / nc;
        } else {
            env = 0.0, genv = 0.0;
        }
    } else if (f.envelope == ENV_FLATTOP) {
        if (fabs(phase) > PI * (nc + 1.0)) {
            env = 0.0, genv = 0.0;
        } else if (fabs(phase) > PI * (nc - 1.0)) {
            double arg = 0.25 * (fabs(phase) - (nc - 1.0) * PI);
            env = powi(cos(arg), 4);
            genv = kk * dsign(phase) * sin(arg) * powi(cos(arg), 3);
        } else {
            env = 1.0, genv = 0.0;
        }
    } else {
        double tau = f.omega * f.duration;
        double e = exp(-4.0 * LN_2 * phase * phase / (tau * tau));
        env = e;
        genv = 8.0 * LN_2 * kk * phase * e / (tau * tau);
    }
    double t = beam * genv + gb2 * env;
    return d4{-t, -(gb0 * env), -(gb1 * env), -t};
}

// focused_laser.rs:80-161 with the Gaussian envelope: <a^2> and its raised
// four-gradient from one exponential (the beam's and the envelope's
// factors combined) and one division, with the reciprocals of the waist,
// Rayleigh range and duration formed on the host.  The same quantities as
// lma_a_sqd and lma_grad_a_sqd to a few ulps.
__device__ __forceinline__ double lma_fg_a_sqd(const FieldParams& f, d4 r) {
    double zz = r.z * f.inv_zr;
    double iw = 1.0 / (1.0 + zz * zz);
    double rho2 = (r.x * r.x + r.y * r.y) * f.inv_w2;
    double phase = phase_of(f, r);
    return f.asq0 * exp(-2.0 * rho2 * iw - f.env_c * (phase * phase)) * iw;
}

__device__ __forceinline__ d4 lma_fg_grad_a_sqd(const FieldParams& f, d4 r) {
    double zz = r.z * f.inv_zr;
    double iw = 1.0 / (1.0 + zz * zz);
    double rho2 = (r.x * r.x + r.y * r.y) * f.inv_w2;
    double phase = phase_of(f, r);
    double be = f.asq0 * exp(-2.0 * rho2 * iw - f.env_c * (phase * phase)) * iw;  // beam * envelope
    double gx = -4.0 * be * r.x * f.inv_w2 * iw;
    double gy = -4.0 * be * r.y * f.inv_w2 * iw;
    double gz = (2.0 * be * r.z * (f.inv_zr * f.inv_zr) * iw) * (2.0 * rho2 * iw - 1.0);
    double t = be * (2.0 * f.k * f.env_c * phase) + gz;
    return d4{-t, -gx, -gy, -t};
}

__device__ __forceinline__ bool lma_fast_gauss(const FieldParams& f) {
    return f.model == M_FOCUSED_LASER && f.envelope == ENV_GAUSSIAN;
}

// <a^2> and its gradient for any LMA model
__device__ __forceinline__ double lma_asq(const FieldParams& f, d4 r) {
    return lma_fast_gauss(f) ? lma_fg_a_sqd(f, r) : lma_a_sqd(f, r);
}
__device__ __forceinline__ d4 lma_grad(const FieldParams& f, d4 r) {
    return lma_fast_gauss(f) ? lma_fg_grad_a_sqd(f, r) : lma_grad_a_sqd(f, r);
}

// A whole LMA step lies where <a^2> < 2^-60 (f.lma_cut): either it ends
// before the pulse (the phase k(t - z) of a massive particle only grows, by
// at most 2 k c dt per step) or it starts after it.
__device__ __forceinline__ bool lma_step_field_free(const FieldParams& f, d4 r, double dt) {
    if (f.lma_cut <= 0.0) return false;
    double phase = phase_of(f, r);
    return phase + 2.0 * f.omega * dt + 1.0 < -f.lma_cut || phase > f.lma_cut;
}

// lma_push where <a^2> and its gradient are below 2^-60: the ponderomotive
// kick and the radiation-reaction terms (all proportional to them) are
// below an ulp of u, and 1 + <a^2> rounds to 1, so u keeps its spatial part,
// gamma is recomputed from it and the particle drifts two half steps, with
// lma_push's own arithmetic.  The work done, also proportional to <a^2>, is
// taken as zero.
__device__ __forceinline__ void lma_push_field_free(d4 r0, d4 u0, double dt, d4* r_out, d4* u_out, double* dt_out) {
    double dtau = dt / u0.t;
    double h = 0.5 * SPEED_OF_LIGHT * dtau;
    d4 r = d4{r0.t + h * u0.t, r0.x + h * u0.x, r0.y + h * u0.y, r0.z + h * u0.z};
    double dt_actual = 0.5 * u0.t * dtau;
    d4 u = u0;
    r = d4{r.t + h * u.t, r.x + h * u.x, r.y + h * u.y, r.z + h * u.z};
    dt_actual = dt_actual + 0.5 * u.t * dtau;
    double b = 1.0;
    u.t = sqrt(b + u.x * u.x + u.y * u.y + u.z * u.z);
    *r_out = r;
    *u_out = u;
    *dt_out = dt_actual;
}

// plane_wave.rs:196-249 == focused_laser.rs:205-258: proper-time leapfrog
// of the ponderomotive equation of motion, with cycle-averaged LL.
__device__ __forceinline__ void lma_push(const FieldParams& f, d4 r0, d4 u0, double rqm, double dt, int eqn,
                                         d4* r_out, d4* u_out, double* dt_out, double* dwork) {
    double dtau = dt / u0.t;
    // charge in units of e: exactly -1 or +1 for electrons and positrons
    constexpr double RQM_E = ELECTRON_CHARGE / ELECTRON_MASS;
    double q = rqm == RQM_E ? 1.0 : rqm == -RQM_E ? -1.0 : rqm / RQM_E;
    double scale = q * q;
    bool rr = eqn == EQN_LL;
    double kk = f.k;
    auto kdot = [&](d4 u) { return kk * u.t - kk * u.z; };
    d4 u_mid = d4{0.0, 0.0, 0.0, 0.0};
    if (rr) {
        d4 g4 = lma_grad(f, r0);
        double fs = 0.5 * SPEED_OF_LIGHT * scale;
        double eta = SPEED_OF_LIGHT * COMPTON_TIME * kdot(u0);
        double llc = scale * scale * (-2.0 * ALPHA_FINE * lma_asq(f, r0) * eta * eta) / (3.0 * COMPTON_TIME);
        u_mid = d4{u0.t + 0.5 * (fs * g4.t + llc * u0.t) * dtau, u0.x + 0.5 * (fs * g4.x + llc * u0.x) * dtau,
                   u0.y + 0.5 * (fs * g4.y + llc * u0.y) * dtau, u0.z + 0.5 * (fs * g4.z + llc * u0.z) * dtau};
    }
    double h = 0.5 * SPEED_OF_LIGHT * dtau;
    d4 r = d4{r0.t + h * u0.t, r0.x + h * u0.x, r0.y + h * u0.y, r0.z + h * u0.z};
    double dt_actual = 0.5 * u0.t * dtau;
    d4 g4 = lma_grad(f, r);
    double fs = 0.5 * SPEED_OF_LIGHT * scale;
    d4 fv = d4{fs * g4.t, fs * g4.x, fs * g4.y, fs * g4.z};
    d4 gv = d4{0.0, 0.0, 0.0, 0.0};
    double asq_mid = 0.0;
    if (rr) {
        double eta = SPEED_OF_LIGHT * COMPTON_TIME * kdot(u_mid);
        asq_mid = lma_asq(f, r);
        double llc = scale * scale * (-2.0 * ALPHA_FINE * asq_mid * eta * eta) / (3.0 * COMPTON_TIME);
        gv = d4{llc * u_mid.t, llc * u_mid.x, llc * u_mid.y, llc * u_mid.z};
    }
    d4 u = d4{u0.t + (fv.t + gv.t) * dtau, u0.x + (fv.x + gv.x) * dtau, u0.y + (fv.y + gv.y) * dtau,
              u0.z + (fv.z + gv.z) * dtau};
    if (rr) {
        double eta = SPEED_OF_LIGHT * COMPTON_TIME * kdot(u_mid);
        double delta = f.circular ? 1.0 : 0.75;
        double llw = 2.0 * ALPHA_FINE * f.omega * eta * delta * (asq_mid * asq_mid) / 3.0;
        *dwork = (fv.t + llw) * dtau;
    } else {
        *dwork = fv.t * dtau;
    }
    r = d4{r.t + h * u.t, r.x + h * u.x, r.y + h * u.y, r.z + h * u.z};
    dt_actual = dt_actual + 0.5 * u.t * dtau;
    double b = 1.0 + lma_asq(f, r);
    u.t = sqrt(b + u.x * u.x + u.y * u.y + u.z * u.z);
    *r_out = r;
    *u_out = u;
    *dt_out = dt_actual;
}

}  // namespace ptg
