// Primary beams on the device: BeamBuilder::build (particle/builder.rs:
// 173-219) with GammaDistribution::sample and RadialDistribution::sample
// (particle/dstr.rs:27-225).  One thread per primary; particle i draws from
// its own Philox stream, in the reference's order within a particle (energy
// and longitudinal offset, the two divergence angles, the transverse
// position), so a beam does not depend on the launch shape.
#include "ptg_launch.h"
#include "ptg_math.cuh"

namespace ptg {

// Standard normal by Box-Muller from two uniforms of the particle's stream.
__device__ __forceinline__ double beam_normal(Draws& rng) {
    double u1 = rng.next(), u2 = rng.next();
    return sqrt(-2.0 * log(1.0 - u1)) * cos(2.0 * PI * u2);
}

// dstr.rs:161-225: (gamma, dz); false if a rejection loop ran out.
__device__ __forceinline__ bool beam_gamma(const BeamArgs& b, Draws& rng, double* gamma, double* dz) {
    if (b.gamma_dstr == 0) {
        for (int it = 0; it < REJECTION_CAP; ++it) {
            double n0 = beam_normal(rng), n1 = beam_normal(rng);
            double n2 = b.rho * n0 + sqrt(1.0 - b.rho * b.rho) * n1;
            double g = b.gamma_mean + b.gamma_sigma * n2;
            if (g > 1.0) {
                *gamma = g;
                *dz = b.sigma_z * n0;
                return true;
            }
        }
        return false;
    }
    if (b.gamma_dstr == 1) {
        // incoherent bremsstrahlung spectrum 4/(3x) - 4/3 + x on [x_min, 1]
        double x_min = b.gamma_min / b.gamma_max;
        double y_max = 4.0 / (3.0 * x_min) - 4.0 / 3.0 + x_min;
        for (int it = 0; it < REJECTION_CAP; ++it) {
            double x = x_min + (1.0 - x_min) * rng.next();
            double u = rng.next();
            double y = 4.0 / (3.0 * x) - 4.0 / 3.0 + x;
            if (u <= y / y_max) {
                *gamma = x * b.gamma_max;
                *dz = b.sigma_z * beam_normal(rng);
                return true;
            }
        }
        return false;
    }
    // tabulated spectrum: correlated normals, then N(0,1) -> U(0,1) with the
    // reference's tanh form of erf (dstr.rs:206-212), then the CDF's inverse
    double n0 = beam_normal(rng);
    double n1 = b.rho * n0 + sqrt(1.0 - b.rho * b.rho) * beam_normal(rng);
    double x = n1 / SQRT_2;
    double u1 = 0.5 * (1.0 + tanh(167.0 * x / 148.0 + 11.0 * x * x * x / 109.0));
    *dz = b.sigma_z * n0;
    return pw_invert(b.custom_cdf, b.custom_len, false, u1, gamma);
}

// dstr.rs:27-51: (x, y); false if the truncated normal ran out.
__device__ __forceinline__ bool beam_radial(const BeamArgs& b, Draws& rng, double* x, double* y) {
    if (b.radial_dstr == 0) {
        *x = b.sigma_x * beam_normal(rng);
        *y = b.sigma_y * beam_normal(rng);
        return true;
    }
    if (b.radial_dstr == 1) {
        for (int it = 0; it < REJECTION_CAP; ++it) {
            double xx = b.sigma_x * beam_normal(rng), yy = b.sigma_y * beam_normal(rng);
            if (xx * xx / (b.x_max * b.x_max) + yy * yy / (b.y_max * b.y_max) <= 1.0) {
                *x = xx, *y = yy;
                return true;
            }
        }
        return false;
    }
    double r = b.r_max * sqrt(rng.next());
    double th = 2.0 * PI * rng.next();
    *x = r * cos(th), *y = r * sin(th);
    return true;
}

__global__ void k_build_beam(BeamArgs b, unsigned long long n, unsigned long long seed, unsigned long long first_id,
                             int* species, double* r, double* u, double* pol, double* weight, unsigned long long* id,
                             unsigned long long* parent_id, unsigned long long* errors) {
    unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    Draws rng;
    rng.begin(seed, mix64(first_id + i + 0xB5AD4ECEDA1CE2A9ull), 0);
    double gamma = 1.0, dz = 0.0, x = 0.0, y = 0.0;
    bool ok = beam_gamma(b, rng, &gamma, &dz);
    double um = b.species == 2 ? -gamma : -sqrt(gamma * gamma - 1.0);
    double theta_x = b.angle + b.rms_div * beam_normal(rng);
    double theta_y = b.rms_div * beam_normal(rng);
    double ux = um * sin(theta_x) * cos(theta_y), uy = um * sin(theta_y), uz = um * cos(theta_x) * cos(theta_y);
    double rx = b.cos_p * ux - b.sin_p * uy, ry = b.sin_p * ux + b.cos_p * uy;
    double usq = rx * rx + ry * ry + uz * uz;
    double u0 = b.species == 2 ? sqrt(usq) : sqrt(1.0 + usq);
    double t, z;
    if (b.off_z >= 0.0) {
        t = -b.initial_z;
        z = b.initial_z + b.off_z + dz;
    } else {
        t = -b.initial_z - fabs(b.off_z);
        z = b.initial_z + dz;
    }
    ok = beam_radial(b, rng, &x, &y) && ok;
    x += b.off_x, y += b.off_y;
    // rotate_around_y(angle), then rotate_around_z(plane)
    double x1 = b.cos_a * x + b.sin_a * z, z1 = b.cos_a * z - b.sin_a * x;
    double x2 = b.cos_p * x1 - b.sin_p * y, y2 = b.sin_p * x1 + b.cos_p * y;
    if (species) species[i] = b.species;
    if (r) r[4 * i] = t, r[4 * i + 1] = x2, r[4 * i + 2] = y2, r[4 * i + 3] = z1;
    if (u) u[4 * i] = u0, u[4 * i + 1] = rx, u[4 * i + 2] = ry, u[4 * i + 3] = uz;
    if (pol)
        for (int k = 0; k < 4; ++k) pol[4 * i + k] = b.pol[k];
    if (weight) weight[i] = b.weight;
    if (id) id[i] = first_id + i;
    if (parent_id) parent_id[i] = first_id + i;
    if (!ok) atomicAdd(errors, 1ull);
}

cudaError_t launch_build_beam(const BeamArgs& b, unsigned long long n, unsigned long long seed,
                              unsigned long long first_id, int* species, double* r, double* u, double* pol,
                              double* weight, unsigned long long* id, unsigned long long* parent_id,
                              unsigned long long* errors, cudaStream_t s) {
    k_build_beam<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(b, n, seed, first_id, species, r, u, pol, weight, id,
                                                             parent_id, errors);
    return cudaGetLastError();
}

}  // namespace ptg
