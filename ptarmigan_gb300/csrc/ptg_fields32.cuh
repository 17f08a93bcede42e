// FP32 evaluation of the LCFA fields for the per-step rates.
//
// The emission and pair-creation probabilities of a step need the quantum
// parameter chi only to the precision of the rate tables, so these
// functions evaluate E and B in FP32 (FP32 pipes are ~64x the FP64 rate on
// GB300).  The carrier phase k.r (hundreds of radians) is reduced modulo
// 2 pi in FP64 first, so the FP32 sine and cosine see an argument in
// [-pi, pi].  Fields are returned normalised: e = E / E0, b = c B / E0.
// Positions, momenta and the push stay FP64 (ptg_fields.cuh), and an event
// recomputes its fields in FP64 before sampling.
#pragma once
#include "ptg_fields.cuh"
#include "ptg_lcfa.cuh"

namespace ptg {

struct f3 {
    float x, y, z;
};
__device__ __forceinline__ f3 f3add(f3 a, f3 b) { return f3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 f3scale(float s, f3 a) { return f3{s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ float f3dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 f3cross(f3 a, f3 b) { return f3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }

struct cf {
    float re, im;
};
__device__ __forceinline__ cf cfmul(cf a, cf b) { return cf{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ __forceinline__ cf cfadd(cf a, cf b) { return cf{a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ cf cfs(float s, cf a) { return cf{s * a.re, s * a.im}; }
__device__ __forceinline__ cf cfadds(float s, cf a) { return cf{s + a.re, a.im}; }

// phase reduced to [-pi, pi] in FP64
__device__ __forceinline__ float reduced_phase(double ph) {
    const double TWO_PI = 6.283185307179586476925;
    return (float)(ph - TWO_PI * rint(ph * (1.0 / TWO_PI)));
}

// Salamin beam (fast_focused_laser.rs:59-111) in FP32, normalised to E0.
// (cr, sr) rotate by the polarisation angle.  Returns false, with zero
// fields, where the transverse Gaussian exp(-rho^2 / (1 + z^2)) is below
// e^-110: there the FP32 factor is an exact zero and so would every field
// component be (a particle far off axis, e.g. a photon emitted at a large
// angle, then steps without evaluating the beam).
__device__ __forceinline__ bool ffl_beam32(const FieldParams& f, d4 r, double cr, double sr, float c, float s,
                                           f3* reE, f3* imE, f3* reB, f3* imB) {
    double rx = cr * r.x + sr * r.y;
    double ry = cr * r.y - sr * r.x;
    float x = (float)(rx * f.inv_waist), y = (float)(ry * f.inv_waist), z = (float)(r.z * f.inv_zr);
    float rho2 = x * x + y * y;
    float e = f.eps32, e2 = e * e, e3 = e2 * e, e4 = e2 * e2;
    float den = 1.0f / (1.0f + z * z);
    cf fc = cf{den, z * den};
    if (fc.re * rho2 > 110.0f) {
        *reE = *imE = *reB = *imB = f3{0.0f, 0.0f, 0.0f};
        return false;
    }
    float ex = expf(-fc.re * rho2);
    float ph = reduced_phase(f.k * r.t - f.k * r.z);
    float sn, cs;
    sincosf(ph - fc.im * rho2, &sn, &cs);
    cf pre = cfmul(fc, cf{ex * cs, ex * sn});
    cf f2 = cfmul(fc, fc), f3c = cfmul(f2, fc), f4 = cfmul(f2, f2);
    float rho4 = rho2 * rho2, rho6 = rho4 * rho2, rho8 = rho4 * rho4;
    cf t2 = cfadds(x * x, cfs(-rho4 * 0.25f, fc));
    cf t4 = cfadds(0.125f, cfs(-rho2 * 0.25f, fc));
    t4 = cfadd(t4, cfs(x * x * rho2 - rho4 * 0.0625f, f2));
    t4 = cfadd(t4, cfs(rho4 * (-x * x - 0.5f * rho2) * 0.25f, f3c));
    t4 = cfadd(t4, cfs(rho8 * 0.03125f, f4));
    cf Ex = cfadds(1.0f, cfadd(cfs(e2, cfmul(f2, t2)), cfs(e4, cfmul(f2, t4))));
    Ex = cfmul(pre, Ex);
    Ex = cf{Ex.im, -Ex.re};
    cf ty = cfadd(cfs(e2 * x * y, f2), cfs(e4 * x * y * rho2, cfmul(f4, cfadds(1.0f, cfs(-rho2 * 0.25f, fc)))));
    cf Ey = cfmul(pre, ty);
    Ey = cf{Ey.im, -Ey.re};
    cf tz = cfadds(-0.5f, cfadd(cfs(rho2, fc), cfs(-rho4 * 0.25f, f2)));
    cf Ez = cfmul(pre, cfadd(cfs(e * x, fc), cfs(e3 * x, cfmul(f2, tz))));
    cf b2 = cfs(rho2 * 0.5f, cfadds(1.0f, cfs(-rho2 * 0.5f, fc)));
    cf b4 = cfadds(-1.0f, cfs(2.0f * rho2, fc));
    b4 = cfadd(b4, cfs(2.5f * rho4, f2));
    b4 = cfadd(b4, cfs(-2.0f * rho6, f3c));
    b4 = cfadd(b4, cfs(0.25f * rho8, f4));
    cf By = cfadds(1.0f, cfadd(cfs(e2, cfmul(f2, b2)), cfs(e4 * 0.125f, cfmul(f2, b4))));
    By = cfmul(pre, By);
    By = cf{By.im, -By.re};
    cf bz = cfadds(1.0f, cfadd(cfs(rho2, fc), cfs(-rho4 * 0.5f, f2)));
    cf Bz = cfmul(pre, cfadd(cfs(e * y, fc), cfs(e3 * y * 0.5f, cfmul(f2, bz))));
    *reE = f3{c * Ex.re - s * Ey.re, c * Ey.re + s * Ex.re, Ez.re};
    *imE = f3{c * Ex.im - s * Ey.im, c * Ey.im + s * Ex.im, Ez.im};
    *reB = f3{-s * By.re, c * By.re, Bz.re};
    *imB = f3{-s * By.im, c * By.im, Bz.im};
    return true;
}

// Normalised fields at r (e = E/E0, b = cB/E0).  Returns false where the
// envelope is below the field-free cut (e = b = 0).
__device__ __forceinline__ bool lcfa_fields32(const FieldParams& f, d4 r, f3* e, f3* b) {
    double phase = phase_of(f, r);
    if (f.model == M_FAST_PLANE_WAVE) {
        // fast_plane_wave.rs:121-195 divided by the amplitude
        float delta = f.circular ? 1.0f : 0.0f;
        double psi = phase * (1.0 + f.chirp_b * phase);
        float dpsi = (float)(1.0 + 2.0 * f.chirp_b * phase);
        double nc = f.n_cycles;
        float env, denv;
        if (f.envelope == ENV_COS2) {
            if (fabs(phase) < nc * PI) {
                float c = cosf((float)(phase / (2.0 * nc)));
                env = c * c;
                denv = -sinf((float)(phase / nc)) / (float)(2.0 * nc);
            } else {
                env = 0.0f, denv = 0.0f;
            }
        } else if (f.envelope == ENV_FLATTOP) {
            if (fabs(phase) > PI * (nc + 1.0)) {
                env = 0.0f, denv = 0.0f;
            } else if (fabs(phase) > PI * (nc - 1.0)) {
                float arg = (float)(0.25 * (fabs(phase) - (nc - 1.0) * PI));
                float c = cosf(arg);
                env = c * c;
                denv = -(phase < 0.0 ? -1.0f : 1.0f) * 0.25f * sinf(2.0f * arg);
            } else {
                env = 1.0f, denv = 0.0f;
            }
        } else {
            double q = phase / (PI * nc);
            env = exp2f((float)(-0.5 * q * q));
            denv = (float)(-LN_2 * phase / ((PI * nc) * (PI * nc))) * env;
        }
        float sp, cp;
        sincosf(reduced_phase(psi), &sp, &cp);
        float dax = sp * denv + cp * dpsi * env;
        float day = delta * (cp * denv - sp * dpsi * env);
        // E = -amp (dax, day, 0); c B = amp (day, -dax, 0); E0 := amp k-normalised
        f3 ev = f3{-dax, -day, 0.0f};
        f3 bv = f3{day, -dax, 0.0f};
        float c = (float)f.cos_pa, s = (float)f.sin_pa;
        *e = f3{c * ev.x - s * ev.y, c * ev.y + s * ev.x, 0.0f};
        *b = f3{c * bv.x - s * bv.y, c * bv.y + s * bv.x, 0.0f};
        return true;
    }
    if (f.env_cut > 0.0 && fabs(phase) > f.env_cut) {
        *e = f3{0.f, 0.f, 0.f};
        *b = f3{0.f, 0.f, 0.f};
        return false;
    }
    // fast_focused_laser.rs:123-151 envelope, in FP32 after an FP64 argument
    float env, denv;
    if (f.envelope == ENV_GAUSSIAN) {
        float q = (float)(phase * f.inv_tau);
        env = expf(-2.0f * (float)LN_2 * q * q);
        denv = (-4.0f * (float)LN_2 * f.inv_tau32) * q * env;
    } else {
        double de, dd;
        ffl_envelope(f, phase, &de, &dd);
        env = (float)de, denv = (float)dd;
    }
    f3 reE, imE, reB, imB;
    if (!ffl_beam32(f, r, f.cos_pa, f.sin_pa, f.cos_pa32, f.sin_pa32, &reE, &imE, &reB, &imB)) {
        *e = f3{0.f, 0.f, 0.f};
        *b = f3{0.f, 0.f, 0.f};
        return false;
    }
    f3 ee = f3add(f3scale(env, reE), f3scale(denv, imE));
    f3 bb = f3add(f3scale(env, reB), f3scale(denv, imB));
    if (f.circular) {
        d4 rp = d4{r.t, r.y, -r.x, r.z};
        ffl_beam32(f, rp, 1.0, 0.0, 1.0f, 0.0f, &reE, &imE, &reB, &imB);
        f3 ey = f3add(f3scale(env, imE), f3scale(-denv, reE));
        f3 by = f3add(f3scale(env, imB), f3scale(-denv, reB));
        ee = f3add(ee, f3{-ey.y, ey.x, ey.z});
        bb = f3add(bb, f3{-by.y, by.x, by.z});
    }
    *e = ee;
    *b = bb;
    return true;
}

// Field scale of lcfa_fields32 in V/m: FastFocusedLaser's E0, or the plane
// wave's amplitude m c^2 k a0 / e.
__device__ __forceinline__ double field_scale(const FieldParams& f) {
    return f.model == M_FAST_PLANE_WAVE ? f.amp : f.E0;
}

// FP32 quantum synchrotron rate (lcfa/photon_emission/mod.rs:13-33), per second.
// `lnh`: PTG_LCFA_LN_H_CHI_TABLE in FP32.
__device__ __forceinline__ float lcfa_photon_rate32(float chi, float gamma, const float (*lnh)[2]) {
    float h;
    if (chi < 0.01f) {
        h = 5.0f * (float)FRAC_PI_3 * (1.0f - 8.0f * chi / (5.0f * (float)SQRT_3));
    } else if (chi >= 100.0f) {
        float c = cbrtf(chi);
        h = -1019.4661473121777f + 1786.716527650374f * c * c;
        h = 1750.6263395722715f + c * c * h;
        h = -2260.1819695887225f + c * h;
        h = 0.00296527643253334f * h / (chi * chi);
    } else {
        float index = (logf(chi) - lnh[0][0]) / (float)PTG_LCFA_PH_DELTA_LN_CHI;
        int i = (int)floorf(index);
        i = i < 0 ? 0 : (i > 39 ? 39 : i);
        float w = index - (float)i;
        float ln_h = (1.0f - w) * lnh[i][1] + w * lnh[i + 1][1];
        h = expf(ln_h);
    }
    return (float)(SQRT_3 * ALPHA_FINE / (2.0 * PI * COMPTON_TIME)) * chi * h / gamma;
}

// FP32 mean of T_par and T_perp (lcfa/pair_creation/mod.rs:13-40): the
// unpolarised Breit-Wheeler auxiliary function.
// `T`: PTG_LCFA_LN_T_CHI_TABLE in FP32.
__device__ __forceinline__ float lcfa_t_mean32(float chi, const float (*T)[3]) {
    const float D = (float)PTG_LCFA_PAIR_DELTA_LN_CHI;
    if (chi <= 0.01f) return 0.0f;
    if (chi < 1.0f) {
        float lc = logf(chi);
        int i = (int)((lc - T[0][0]) / D);
        i = i < 0 ? 0 : (i > 79 ? 79 : i);
        float e0 = expf(T[i][0]), e1 = expf(T[i + 1][0]);
        float dx = (chi - e0) / (e1 - e0);
        float par = (1.0f - dx) / T[i][1] + dx / T[i + 1][1];
        float perp = (1.0f - dx) / T[i][2] + dx / T[i + 1][2];
        return 0.5f * (expf(1.0f / par) + expf(1.0f / perp));
    }
    if (chi < 100.0f) {
        float lc = logf(chi);
        int i = (int)((lc - T[0][0]) / D);
        i = i < 0 ? 0 : (i > 79 ? 79 : i);
        float dx = (lc - T[i][0]) / D;
        return 0.5f * (expf((1.0f - dx) * T[i][1] + dx * T[i + 1][1]) +
                       expf((1.0f - dx) * T[i][2] + dx * T[i + 1][2]));
    }
    float c = cbrtf(chi);
    return 0.5f * ((0.3036898468348568f + 0.4555347702522852f) / c - 4.0f / (3.0f * chi));
}

}  // namespace ptg
