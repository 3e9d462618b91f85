// Device functions shared by the HBM-streaming and the shared-memory resident sweep kernels.
// Both kernels call exactly these functions with the same operands, so the two paths
// produce bit-identical chains for the same Philox counters.
#pragma once
#include "nmmc_internal.h"

namespace nmmc {

constexpr float kPi = 3.14159265358979f;

// Compact index, in the other colour's plane, of the neighbour of (x,y,z) in direction k
// (+x,-x,+y,-y,+z,-z), or -1 when the neighbour falls off an open boundary.
template <bool PERIODIC>
__device__ __forceinline__ int nb_compact(const DevModel& m, int x, int y, int z, int k) {
    int nx = x, ny = y, nz = z;
    switch (k) {
        case 0: nx++; break;
        case 1: nx--; break;
        case 2: ny++; break;
        case 3: ny--; break;
        case 4: nz++; break;
        default: nz--; break;
    }
    if (PERIODIC) {
        const int e = m.edge;
        nx = (nx == e) ? 0 : (nx < 0 ? e - 1 : nx);
        ny = (ny == e) ? 0 : (ny < 0 ? e - 1 : ny);
        if (k >= 4) nz = (nz == e) ? 0 : (nz < 0 ? e - 1 : nz);
    } else {
        if (nx < 0 || nx >= m.edge || ny < 0 || ny >= m.edge || nz < 0 || nz >= m.lz) return -1;
    }
    return (nz * m.ly + ny) * m.hx + (nx >> 1);
}

// Site of compact index i in colour `colour`.
template <int DIM>
__device__ __forceinline__ void decode_site(const DevModel& m, int i, int colour, int& x, int& y,
                                            int& z) {
    int row = i / m.hx;
    int h = i - row * m.hx;
    if (DIM == 3) {
        z = row / m.ly;
        y = row - z * m.ly;
    } else {
        z = 0;
        y = row;
    }
    x = 2 * h + ((y + z + colour) & 1);
}

// Philox4x32-10 with the round keys read from the kernel parameters (same values as
// nmmc_philox with key (key0, key1); the key schedule costs no instructions here). WIDE
// forms each round's products as one 32 x 32 -> 64-bit multiply instead of separate low and
// high halves: the same words, and measured 0.6 % faster in the HBM half-sweep but 0.7 %
// slower in the shared-memory resident kernel, so each kernel picks its form.
template <bool WIDE = false>
__device__ __forceinline__ nmmc_u4 philox_rk(const DevModel& m, uint32_t c0, uint32_t c1, uint32_t c2,
                                             uint32_t c3) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t lo0, hi0, lo1, hi1;
        if (WIDE) {
            const unsigned long long p0 = (unsigned long long)c0 * 0xD2511F53u;
            const unsigned long long p1 = (unsigned long long)c2 * 0xCD9E8D57u;
            lo0 = (uint32_t)p0;
            hi0 = (uint32_t)(p0 >> 32);
            lo1 = (uint32_t)p1;
            hi1 = (uint32_t)(p1 >> 32);
        } else {
            lo0 = 0xD2511F53u * c0;
            hi0 = __umulhi(0xD2511F53u, c0);
            lo1 = 0xCD9E8D57u * c2;
            hi1 = __umulhi(0xCD9E8D57u, c2);
        }
        uint32_t n0 = hi1 ^ c1 ^ m.rk0[r];
        uint32_t n2 = hi0 ^ c3 ^ m.rk1[r];
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
    }
    return nmmc_u4{c0, c1, c2, c3};
}

template <bool WIDE = false>
__device__ __forceinline__ nmmc_u4 sweep_draw(const DevModel& m, uint32_t box, unsigned long long s,
                                              uint32_t chain) {
    return philox_rk<WIDE>(m, box, (uint32_t)s, (uint32_t)(s >> 32) | (NMMC_STREAM_SWEEP << 28), chain);
}

// DMI structure of a model, fixed for every sweep kernel so that all paths compute the local
// field with the same operations (and so produce the same chain):
//   0: no DMI; 1: any per-direction DMI vectors;
//   2: +-axis pairs with J(+a) == J(-a) and Ds(-a) == -Ds(+a): field J(s+ + s-) + (s+ - s-) x Ds(+a);
//   3: as 2, with each Ds(+a) along its own axis a (bulk / Bloch DMI).
enum { kDmiNone = 0, kDmiGeneral = 1, kDmiPairs = 2, kDmiAxial = 3 };

// Local field of the sweep: H + sum_k J_k s_k + s_k x Ds_k (FP32).
template <int NDIR, int DK>
__device__ __forceinline__ void heis_field(const DevModel& m, const float* nx, const float* ny,
                                           const float* nz, float4 p, float& hx, float& hy,
                                           float& hz) {
    hx = p.y;
    hy = p.z;
    hz = p.w;
    if (DK <= kDmiGeneral) {
#pragma unroll
        for (int k = 0; k < NDIR; ++k) {
            hx = fmaf(m.J[k], nx[k], hx);
            hy = fmaf(m.J[k], ny[k], hy);
            hz = fmaf(m.J[k], nz[k], hz);
            if (DK == kDmiGeneral) {
                hx = fmaf(ny[k], m.Ds[k][2], fmaf(-nz[k], m.Ds[k][1], hx));
                hy = fmaf(nz[k], m.Ds[k][0], fmaf(-nx[k], m.Ds[k][2], hy));
                hz = fmaf(nx[k], m.Ds[k][1], fmaf(-ny[k], m.Ds[k][0], hz));
            }
        }
    } else {
#pragma unroll
        for (int a = 0; a < NDIR / 2; ++a) {
            const int kp = 2 * a, km = 2 * a + 1;
            const float sx = nx[kp] + nx[km], sy = ny[kp] + ny[km], sz = nz[kp] + nz[km];
            const float dx = nx[kp] - nx[km], dy = ny[kp] - ny[km], dz = nz[kp] - nz[km];
            hx = fmaf(m.J[kp], sx, hx);
            hy = fmaf(m.J[kp], sy, hy);
            hz = fmaf(m.J[kp], sz, hz);
            if (DK == kDmiPairs) {   // d x Ds(+a)
                hx = fmaf(dy, m.Ds[kp][2], fmaf(-dz, m.Ds[kp][1], hx));
                hy = fmaf(dz, m.Ds[kp][0], fmaf(-dx, m.Ds[kp][2], hy));
                hz = fmaf(dx, m.Ds[kp][1], fmaf(-dy, m.Ds[kp][0], hz));
            } else {                 // Ds(+a) = D_a e_a
                const float D = m.Ds[kp][a];
                if (a == 0) {
                    hy = fmaf(D, dz, hy);
                    hz = fmaf(-D, dy, hz);
                } else if (a == 1) {
                    hx = fmaf(-D, dz, hx);
                    hz = fmaf(D, dx, hz);
                } else {
                    hx = fmaf(D, dy, hx);
                    hy = fmaf(-D, dx, hy);
                }
            }
        }
    }
}

// The DMI part of heis_field's local field alone (the same operations on the same values; the
// compiler shares them with heis_field when both are inlined): sum_k s_k x Ds_k.
template <int NDIR, int DK>
__device__ __forceinline__ void heis_dmi_part(const DevModel& m, const float* nx, const float* ny,
                                              const float* nz, float& hx, float& hy, float& hz) {
    hx = hy = hz = 0.0f;
    if (DK == kDmiNone) return;
    if (DK == kDmiGeneral) {
#pragma unroll
        for (int k = 0; k < NDIR; ++k) {
            hx = fmaf(ny[k], m.Ds[k][2], fmaf(-nz[k], m.Ds[k][1], hx));
            hy = fmaf(nz[k], m.Ds[k][0], fmaf(-nx[k], m.Ds[k][2], hy));
            hz = fmaf(nx[k], m.Ds[k][1], fmaf(-ny[k], m.Ds[k][0], hz));
        }
        return;
    }
#pragma unroll
    for (int a = 0; a < NDIR / 2; ++a) {
        const int kp = 2 * a, km = 2 * a + 1;
        const float dx = nx[kp] - nx[km], dy = ny[kp] - ny[km], dz = nz[kp] - nz[km];
        if (DK == kDmiPairs) {
            hx = fmaf(dy, m.Ds[kp][2], fmaf(-dz, m.Ds[kp][1], hx));
            hy = fmaf(dz, m.Ds[kp][0], fmaf(-dx, m.Ds[kp][2], hy));
            hz = fmaf(dx, m.Ds[kp][1], fmaf(-dy, m.Ds[kp][0], hz));
        } else {
            const float D = m.Ds[kp][a];
            if (a == 0) {
                hy = fmaf(D, dz, hy);
                hz = fmaf(-D, dy, hz);
            } else if (a == 1) {
                hx = fmaf(-D, dz, hx);
                hz = fmaf(D, dx, hz);
            } else {
                hx = fmaf(D, dy, hx);
                hy = fmaf(-D, dx, hy);
            }
        }
    }
}

__device__ __forceinline__ float heis_dE(float hx, float hy, float hz, float sx, float sy, float sz,
                                         float tx, float ty, float tz) {
    return fmaf(hz, sz - tz, fmaf(hy, sy - ty, hx * (sx - tx)));
}

// Uniform proposal on S^2 from two 23-bit uniforms: z uniform in (-1,1), phi in (-pi,pi)
// (Archimedes: z uniform gives equal area). |z| <= 1 - 2^-23, so w = 1 - z^2 (one rounding
// of the exact FMA) is at least 2^-22 - 2^-46 > 0 and the radius sqrt(w) = w rsqrt(w) is
// finite; the hardware reciprocal square root is within a few ulp, so |t| = 1 to about 3e-7.
// This form issues far fewer instructions than the correctly rounded sqrtf.
__device__ __forceinline__ void sphere_proposal(uint32_t r0, uint32_t r1, float& tx, float& ty,
                                                float& tz) {
    tz = fmaf(2.0f, nmmc_u01f(r0), -1.0f);
    float phi = fmaf(2.0f, nmmc_u01f(r1), -1.0f) * kPi;
    float sp, cp;
    __sincosf(phi, &sp, &cp);
    const float w = fmaf(-tz, tz, 1.0f);
    const float rxy = w * rsqrtf(w);
    tx = rxy * cp;
    ty = rxy * sp;
}

// Proposal and Metropolis test for a site whose local field is (hx, hy, hz): returns true
// and the new spin when accepted (Old/lib/state.cpp:182-200).
__device__ __forceinline__ float accept_log(uint32_t r) { return __logf(nmmc_u01f(r)); }

// Metropolis test of a drawn proposal t with log-uniform lu = accept_log(r.z).
__device__ __forceinline__ bool heis_accept(float hx, float hy, float hz, float sx, float sy, float sz,
                                            float4 p, float tx, float ty, float tz, float lu) {
    float dE = heis_dE(hx, hy, hz, sx, sy, sz, tx, ty, tz);
    return (dE <= 0.0f) || (-dE * p.x > lu);
}

__device__ __forceinline__ bool heis_try(float hx, float hy, float hz, float sx, float sy, float sz, float4 p,
                                         nmmc_u4 r, float& tx, float& ty, float& tz) {
    sphere_proposal(r.x, r.y, tx, ty, tz);
    return heis_accept(hx, hy, hz, sx, sy, sz, p, tx, ty, tz, accept_log(r.z));
}


// One Heisenberg Metropolis attempt: returns true and the new spin when accepted.
template <int NDIR, int DK>
__device__ __forceinline__ bool heis_attempt(const DevModel& m, float sx, float sy, float sz,
                                             const float* nx, const float* ny, const float* nz,
                                             float4 p, nmmc_u4 r, float& tx, float& ty, float& tz) {
    float hx, hy, hz;
    heis_field<NDIR, DK>(m, nx, ny, nz, p, hx, hy, hz);
    return heis_try(hx, hy, hz, sx, sy, sz, p, r, tx, ty, tz);
}

// Ising: local field H0 + sum_k J_k s_k; products are exact because s_k is -1, 0 or +1.
template <int NDIR>
__device__ __forceinline__ float ising_field(const DevModel& m, const float* n, float4 p) {
    float h = p.y;
#pragma unroll
    for (int k = 0; k < NDIR; ++k) h = fmaf(m.J[k], n[k], h);
    return h;
}

// Ising proposal and test for local field h, with the reference's proposal: a random +-1,
// not a flip (Old/lib/field_type.cpp:189).
__device__ __forceinline__ bool ising_try(float h, float so, float4 p, nmmc_u4 r, float& t) {
    t = (r.x >> 31) ? 1.0f : -1.0f;
    float dE = h * (so - t);
    return (dE <= 0.0f) || (-dE * p.x > logf(nmmc_u01f(r.y)));
}

// One Ising attempt.
template <int NDIR>
__device__ __forceinline__ bool ising_attempt(const DevModel& m, float so, const float* n, float4 p,
                                              nmmc_u4 r, float& t) {
    return ising_try(ising_field<NDIR>(m, n, p), so, p, r, t);
}

// ------------------------------------------------------------------------------------------
// Observables shared by the measurement kernels and the resident kernel's fused measurement
// (Old/lib/thermodynamics.cpp:71-221).
// ------------------------------------------------------------------------------------------
// Partial sums per chain (or per block of a chain): 0 e = sum_i s_i . sum_j (J s_j + D x s_j),
// 1-3 M, 4-6 subM(0), 7-9 sub4M, 10 solid-angle sum.
constexpr int kNP = 11;

// FP32 atan2 for the solid angles: r = min(|x|,|y|) / max(|x|,|y|) in [0, 1], atan(r) from an
// odd polynomial of degree 15, r P(r^2), whose coefficients were fitted here to atan on [0, 1]
// (near-minimax absolute error 3.7e-8 in exact arithmetic, by iteratively reweighted least
// squares); then the octant reflections atan = pi/2 - atan(1/r) for |y| > |x|, pi - a for
// x < 0 (or -0), and the sign of y. Evaluated in FP32 its error is below 3e-7 rad over the
// arguments a solid angle produces, with no bias; the signed zeros and x = -0 give atan2's
// values (0, -0, +-pi). About half the instructions of atan2f.
__device__ __forceinline__ float atan2_poly(float y, float x) {
    const float ax = fabsf(x), ay = fabsf(y);
    const float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
    const float r = (mx > 0.0f) ? __fdividef(mn, mx) : 0.0f;
    const float t = r * r;
    float p = -0.004054564864481316f;
    p = fmaf(p, t, 0.02186294984597138f);
    p = fmaf(p, t, -0.05591231593978804f);
    p = fmaf(p, t, 0.0964219659851754f);
    p = fmaf(p, t, -0.13908629294723196f);
    p = fmaf(p, t, 0.19946565607923386f);
    p = fmaf(p, t, -0.3332986078147662f);
    p = fmaf(p, t, 0.9999993355780388f);
    float a = r * p;
    if (ay > ax) a = 1.57079632679489662f - a;
    if (__float_as_uint(x) >> 31) a = kPi - a;
    return copysignf(a, y);
}

// FP32 dot product of two spins (symmetric: the same value in either order).
__device__ __forceinline__ float dot3f(float a0, float a1, float a2, float b0, float b1, float b2) {
    return fmaf(a0, b0, fmaf(a1, b1, a2 * b2));
}

// FP32 solid angle (thermodynamics.cpp:200-221). The reference divides both arguments of
// atan2 by rho = 2(1+s1.s2)(1+s1.s3)(1+s2.s3), which is >= 0 for unit spins and leaves the
// angle unchanged whenever rho > 0. In FP32 a pair within ~3.5e-4 rad of antiparallel rounds
// a factor 1+s.s' to exactly 0 (a frequent event at high temperature on large lattices),
// where the FP64 rho is tiny but positive; the rho -> 0+ limit, atan2(cross, dotsum), is
// therefore the FP32 value. The FP64 mode keeps the reference's divisions.
// solid_angle_dots takes the three pair products s1.s2, s1.s3, s2.s3 (dot3f) ready made, so
// that a bond's product can serve both triangles that share it.
__device__ __forceinline__ float solid_angle_dots(float a0, float a1, float a2, float b0, float b1, float b2,
                                                  float c0, float c1, float c2, float s1s2, float s1s3,
                                                  float s2s3) {
    float dotsum = 1.0f + s1s2 + s1s3 + s2s3;
    float x0 = fmaf(a1, c2, -a2 * c1), x1 = fmaf(a2, c0, -a0 * c2), x2 = fmaf(a0, c1, -a1 * c0);
    float cross = fmaf(x0, b0, fmaf(x1, b1, x2 * b2));
    return -atan2_poly(cross, dotsum);
}

__device__ __forceinline__ float solid_angle_f(float a0, float a1, float a2, float b0, float b1, float b2,
                                               float c0, float c1, float c2) {
    return solid_angle_dots(a0, a1, a2, b0, b1, b2, c0, c1, c2, dot3f(a0, a1, a2, b0, b1, b2),
                            dot3f(a0, a1, a2, c0, c1, c2), dot3f(b0, b1, b2, c0, c1, c2));
}

// Observables of one chain from its totals, by one warp (FP64 runs at a small fraction of the
// FP32 rate on this GPU, so the ~250 FP64 instructions of one thread cost microseconds; spread
// over the lanes they are about 50): lane k < kNP - 1 holds total k (0 e, 1-3 M, 4-6 subM(0),
// 7-9 sub4M), qsum is the chain's topological charge (every lane). Writes the NMMC_OBS_N
// observables: E = -H.M - e/2 (the pair sum counts every bond twice), M, |M|, subM, |subM|,
// sub4M, |sub4M|, Q; with `accumulate` adds the sample to the chain's accumulators (n, E, E^2,
// |M|, |M|^2, |M|^4, Q, Q^2). Every lane of the warp must call it.
__device__ __forceinline__ void finalize_chain_warp(double tot_k, int lane, const double* H, double qsum,
                                                    double* o, double* a, int accumulate) {
    const unsigned full = 0xffffffffu;
    // components: observable L <- total L (1-3), L - 1 (5-7), L - 2 (9-11)
    const double comp = __shfl_sync(full, tot_k, (lane - (lane > 4) - (lane > 8)) & 31);
    // norms: lane 8 |subM| (totals 4-6), lane 12 |sub4M| (7-9), every other lane |M| (1-3)
    const int nb = (lane == 8) ? 4 : (lane == 12) ? 7 : 1;
    const double n0 = __shfl_sync(full, tot_k, nb), n1 = __shfl_sync(full, tot_k, nb + 1),
                 n2 = __shfl_sync(full, tot_k, nb + 2);
    const double nrm = sqrt(n0 * n0 + n1 * n1 + n2 * n2);
    const double e = __shfl_sync(full, tot_k, 0), M0 = __shfl_sync(full, tot_k, 1),
                 M1 = __shfl_sync(full, tot_k, 2), M2 = __shfl_sync(full, tot_k, 3);
    const double E = (-H[0] * M0 - H[1] * M1 - H[2] * M2) - 0.5 * e;
    const double am = __shfl_sync(full, nrm, 0);   // lane 0 took the |M| branch
    double val = comp;
    if (lane == NMMC_OBS_E) val = E;
    if (lane == NMMC_OBS_ABSM || lane == NMMC_OBS_ABSSUBM || lane == NMMC_OBS_ABSSUB4M) val = nrm;
    if (lane == NMMC_OBS_QTOT) val = qsum;
    if (lane < NMMC_OBS_N) o[lane] = val;
    if (accumulate && lane < NMMC_ACC_N) {
        const double am2 = am * am;
        double t = 1.0;
        if (lane == 1) t = E;
        if (lane == 2) t = E * E;
        if (lane == 3) t = am;
        if (lane == 4) t = am2;
        if (lane == 5) t = am2 * am2;
        if (lane == 6) t = qsum;
        if (lane == 7) t = qsum * qsum;
        a[lane] += t;
    }
}

}  // namespace nmmc
