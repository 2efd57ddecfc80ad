// device_math.cuh - per-pair and per-tuple arithmetic of the OpenCafeMol
// coarse-grained force field, shared by the plain (global-memory) and the
// batched (shared-memory) engines.
//
// Every function evaluates in FP32.  Forces leave these functions as FP32
// and are accumulated by the callers in 64-bit fixed point (2^32 units per
// kJ/mol/nm), which makes the summation order-independent.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "engine_types.h"
#include "fixed_point.h"

namespace ocm {

// ---------------------------------------------------------------------------
// Fixed-point force accumulation.
// ---------------------------------------------------------------------------
// round(f * 2^32) as int64 without the FP64 pipe (fixed_point.h).
__device__ __forceinline__ unsigned long long to_fixed(float f) { return fixed_from_float(f); }
__device__ __forceinline__ void fixed_add(unsigned long long* p, float f) {
    atomicAdd(p, to_fixed(f));
}

// ---------------------------------------------------------------------------
// Canonical FP32 separation.  d = xj - xi with periodic minimum image; every
// operation is individually rounded (no contraction) so the host-side
// brute-force enumeration can reproduce r^2 bit for bit.
// ---------------------------------------------------------------------------
template <bool PERIODIC>
__device__ __forceinline__ float3 separation(float4 xi, float4 xj, const float3& box,
                                             const float3& inv_box) {
    float dx = __fsub_rn(xj.x, xi.x);
    float dy = __fsub_rn(xj.y, xi.y);
    float dz = __fsub_rn(xj.z, xi.z);
    if (PERIODIC) {
        dx = __fmaf_rn(-box.x, rintf(__fmul_rn(dx, inv_box.x)), dx);
        dy = __fmaf_rn(-box.y, rintf(__fmul_rn(dy, inv_box.y)), dy);
        dz = __fmaf_rn(-box.z, rintf(__fmul_rn(dz, inv_box.z)), dz);
    }
    return make_float3(dx, dy, dz);
}
__device__ __forceinline__ float norm2(float3 d) {
    return __fmaf_rn(d.z, d.z, __fmaf_rn(d.y, d.y, __fmul_rn(d.x, d.x)));
}

// Label test of an interaction-group matrix: 4-bit label per term, 15 = the
// particle takes no part in the term.
__device__ __forceinline__ bool labels_allow(uint32_t li, uint32_t lj, int term,
                                             unsigned long long allow) {
    const uint32_t a = (li >> (4 * term)) & 15u;
    const uint32_t b = (lj >> (4 * term)) & 15u;
    if (a == 15u || b == 15u) return false;
    return (allow >> (a * 8 + b)) & 1ull;
}

struct PairEnergy {
    float exv, dh, ljr, lja;
    __device__ void zero() { exv = dh = ljr = lja = 0.f; }
};

// All pair terms for one (i, j).  Returns the scalar s with F_i = s * (x_i -
// x_j) = -s * d.  excl is the per-term exclusion bits of this pair (bit t set
// = term t excluded), already combined with the interaction-group test.
//
// Terms (reference expressions):
//   EXV  eps (si+sj)^12 (r^-12 - rc^-12)                 ExcludedVolumeForceFieldGenerator.cpp:25-27
//   DH   qi qj k (exp(-r/lD)/r - exp(-rc/lD)/rc)         DebyeHuckelForceFieldGenerator.cpp:54-57
//   LJR  step(t-r) e (4(s^12-s^6)+1), t = 2^(1/6) s      LennardJonesRepulsiveForceFieldGenerator.cpp:35-43
//   LJA  e (step(r-t) 4(s^12-s^6) - step(t-r)) * S(r)    LennardJonesAttractiveForceFieldGenerator.cpp:40-50,114-115
template <int TERMS, bool ENERGY>
__device__ __forceinline__ float pair_scalar(float r2, float4 pi, float4 pj, float4 qi, float4 qj,
                                             uint32_t excl, const PairConsts& pc,
                                             PairEnergy& e) {
    const float rinv = rsqrtf(r2);
    const float r2inv = rinv * rinv;
    float s = 0.f;
    if ((TERMS & kTermEXV) && !(excl & kTermEXV) && r2 < pc.exv_rc2) {
        const float S = pi.x + pj.x;
        const float S2 = S * S;
        const float u = S2 * r2inv;
        const float u3 = u * u * u;
        const float u6 = u3 * u3;
        s += 12.f * pc.exv_eps * u6 * r2inv;
        if (ENERGY) {
            const float w = S2 * pc.exv_inv_rc2;
            const float w3 = w * w * w;
            e.exv += pc.exv_eps * (u6 - w3 * w3);
        }
    }
    // q_i q_j = 0 adds exactly nothing, so skipping it changes no bit
    if ((TERMS & kTermDH) && !(excl & kTermDH) && r2 < pc.dh_rc2 && pi.y != 0.f && pj.y != 0.f) {
        const float r = r2 * rinv;
        const float ex = exp2f(-r * pc.dh_inv_lambda_log2e);
        const float qq = pi.y * pj.y * pc.dh_k;
        s += qq * ex * (pc.dh_inv_lambda + rinv) * r2inv;
        if (ENERGY) e.dh += qq * (ex * rinv - pc.dh_corr);
    }
    // shared sigma: mixing and powers once (same expressions, same bits)
    float sh_sig2 = 0.f, sh_s6 = 0.f, sh_s12 = 0.f;
    if (TERMS & kLJSameSigma) {
        const float sig = 0.5f * (pi.w + pj.w);
        sh_sig2 = sig * sig;
        const float s2 = sh_sig2 * r2inv;
        sh_s6 = s2 * s2 * s2;
        sh_s12 = sh_s6 * sh_s6;
    }
    if ((TERMS & kTermLJR) && !(excl & kTermLJR) && r2 < pc.ljr_rc2) {
        float sig2 = sh_sig2;
        if (!(TERMS & kLJSameSigma)) {
            const float sig = 0.5f * (pi.w + pj.w);
            sig2 = sig * sig;
        }
        if (r2 <= sig2 * kTwoPow1_3) {
            // arithmetic epsilon (LennardJonesRepulsive) or geometric (WCA:
            // p0.z holds sqrt(eps))
            const float eps = pc.ljr_geometric ? pi.z * pj.z : 0.5f * (pi.z + pj.z);
            float s6 = sh_s6, s12 = sh_s12;
            if (!(TERMS & kLJSameSigma)) {
                const float s2 = sig2 * r2inv;
                s6 = s2 * s2 * s2;
                s12 = s6 * s6;
            }
            s += 24.f * eps * (2.f * s12 - s6) * r2inv;
            if (ENERGY) e.ljr += eps * (4.f * (s12 - s6) + 1.f);
        }
    }
    if ((TERMS & kTermLJA) && !(excl & kTermLJA) && r2 < pc.lja_rc2) {
        float sig2 = sh_sig2;
        if (!(TERMS & kLJSameSigma)) {
            const float sig = 0.5f * (qi.y + qj.y);
            sig2 = sig * sig;
        }
        const float eps = 0.5f * (qi.x + qj.x);
        float E, dEdr_over_r;  // dE/dr / r of the unswitched potential
        if (r2 < sig2 * kTwoPow1_3) {
            E = -eps;
            dEdr_over_r = 0.f;
        } else {
            float s6 = sh_s6, s12 = sh_s12;
            if (!(TERMS & kLJSameSigma)) {
                const float s2 = sig2 * r2inv;
                s6 = s2 * s2 * s2;
                s12 = s6 * s6;
            }
            E = 4.f * eps * (s12 - s6);
            dEdr_over_r = -24.f * eps * (2.f * s12 - s6) * r2inv;
        }
        const float r = r2 * rinv;
        if (r > pc.lja_rs) {
            // OpenMM switching function S = 1 - 10x^3 + 15x^4 - 6x^5.
            const float x = (r - pc.lja_rs) * pc.lja_inv_width;
            const float x2 = x * x;
            const float x3 = x2 * x;
            const float sw = 1.f + x3 * (-10.f + x * (15.f - 6.f * x));
            const float dsw = x2 * (-30.f + x * (60.f - 30.f * x)) * pc.lja_inv_width;
            dEdr_over_r = dEdr_over_r * sw + E * dsw * rinv;
            E *= sw;
        }
        s -= dEdr_over_r;
        if (ENERGY) e.lja += E;
    }
    return s;
}

// ---------------------------------------------------------------------------
// Bond-like terms (explicit lists, no cutoff).
// ---------------------------------------------------------------------------
// Harmonic bond 1/2 k (r - r0)^2 (HarmonicBondForceFieldGenerator.cpp:5-10).
// Go 10-12: k (5 (r0/r)^12 - 6 (r0/r)^10) (GoContactForceFieldGenerator.cpp:5-7).
// Gaussian bond: k exp(-(r - v0)^2 / (2 sigma^2))
// (GaussianBondForceFieldGenerator.cpp:5-7).
// `delta` = r^2 - r0^2 (v0^2 for the Gaussian) evaluated without
// cancellation by the caller: all three forces are proportional to it near
// the centre, where an FP32 r - r0 would lose its digits.  For a capped Go
// contact p1 = 1 / cap and p2 = the high part of r0^2.  For a Gaussian
// bond p1 = 1 / (2 sigma^2) and p2 = the high part of v0^2 (v0 enters only
// the r + v0 denominator).  Returns s with F_a = s * (x_a - x_b).
__device__ __forceinline__ float bond_scalar(int kind, float r2, float delta, float p0, float p1,
                                             float p2, float& energy) {
    if (kind == kBondHarmonic) {  // p0 = r0, p1 = k
        const float r = sqrtf(r2);
        const float dr = delta / (r + p0);
        energy = 0.5f * p1 * dr * dr;
        return -p1 * dr / r;
    } else if (kind == kBondGauss) {  // p0 = k, p1 = 1 / (2 sigma^2), p2 ~ v0^2
        const float r = sqrtf(r2);
        const float dr = delta / (r + sqrtf(p2));
        const float e = p0 * expf(-dr * dr * p1);
        energy = e;
        return 2.f * p1 * dr * e / r;
    } else if (kind == kBondGo) {  // Go: p0 = k, p1 = r0;  t^2 - 1 = -delta / r^2
        const float inv = 1.f / r2;
        const float t2 = p1 * p1 * inv;
        const float t10 = t2 * t2 * t2 * t2 * t2;
        energy = p0 * t10 * (5.f * t2 - 6.f);
        return -60.f * p0 * t10 * delta * inv * inv;
    } else {  // capped Go: p0 = k, p1 = u = 1 / cap, p2 ~ r0^2
        // r <= cap r0: the linear continuation k (slope r / r0 + intercept),
        // slope = -60 (u^13 - u^11), intercept = 65 u^12 - 66 u^10, which
        // meets the Go form with its first derivative at r = cap r0
        // (CappedGoContactForceFieldGenerator.cpp); beyond it the Go form.
        if (r2 * p1 * p1 <= p2) {
            const float r = sqrtf(r2), r0 = sqrtf(p2);
            const float u2 = p1 * p1, u10 = u2 * u2 * u2 * u2 * u2;
            const float slope = -60.f * u10 * p1 * (u2 - 1.f);
            energy = p0 * (slope * r / r0 + u10 * (65.f * u2 - 66.f));
            return -p0 * slope / (r0 * r);
        }
        const float inv = 1.f / r2;
        const float t2 = p2 * inv;
        const float t10 = t2 * t2 * t2 * t2 * t2;
        energy = p0 * t10 * (5.f * t2 - 6.f);
        return -60.f * p0 * t10 * delta * inv * inv;
    }
}

// Error-free transforms for float-float ("unevaluated sum") arithmetic.
__device__ __forceinline__ float two_sum(float a, float b, float& err) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    err = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return s;
}
// r^2 - r0^2 for a separation given as dh + dl (|dl| << |dh|), with r0^2 =
// r0sq_hi + r0sq_lo: products split exactly by FMA, sums by TwoSum.
__device__ __forceinline__ float ff_bond_delta(float3 dh, float3 dl, float r0sq_hi, float r0sq_lo) {
    const float px = __fmul_rn(dh.x, dh.x), py = __fmul_rn(dh.y, dh.y), pz = __fmul_rn(dh.z, dh.z);
    const float ex = __fmaf_rn(dh.x, dh.x, -px), ey = __fmaf_rn(dh.y, dh.y, -py),
                ez = __fmaf_rn(dh.z, dh.z, -pz);
    float t1, t2;
    const float s1 = two_sum(px, py, t1);
    const float s2 = two_sum(s1, pz, t2);
    const float lo = t1 + t2 + ex + ey + ez + 2.f * (dh.x * dl.x + dh.y * dl.y + dh.z * dl.z);
    return __fsub_rn(s2, r0sq_hi) + (lo - r0sq_lo);
}
// Separation x_j - x_i of float-float positions: hi part exact by TwoSum.
__device__ __forceinline__ void ff_sep(float4 hi_i, float3 lo_i, float4 hi_j, float3 lo_j,
                                       float3& dh, float3& dl) {
    float e;
    dh.x = two_sum(hi_j.x, -hi_i.x, e);
    dl.x = e + (lo_j.x - lo_i.x);
    dh.y = two_sum(hi_j.y, -hi_i.y, e);
    dl.y = e + (lo_j.y - lo_i.y);
    dh.z = two_sum(hi_j.z, -hi_i.z, e);
    dl.z = e + (lo_j.z - lo_i.z);
}

// Flexible-local angle (FlexibleLocalAngleForceFieldGenerator.cpp:21-25):
// E = k (spline(theta) - Emin + step(tmin-theta)(30 (tmin-theta) + y0)
//                             + step(theta-tmax)(30 (theta-tmax) + y9)),
// spline = natural cubic spline through 10 equidistant nodes, 0 outside.
// Writes forces on the three particles.
__device__ __forceinline__ void fla_forces(float3 u, float3 v, float kk, const FlaTable& t,
                                           float3& f1, float3& f3, float& energy) {
    // u = x1 - x2, v = x3 - x2
    const float3 n = make_float3(u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x);
    const float nn = fmaxf(norm2(n), 1e-30f);
    const float nlen = sqrtf(nn);
    const float dot = u.x * v.x + u.y * v.y + u.z * v.z;
    const float theta = atan2f(nlen, dot);
    float S = 0.f, dS = 0.f;
    if (theta < t.theta_min) {
        S = 30.f * (t.theta_min - theta) + t.y[0];
        dS = -30.f;
    } else if (theta > t.theta_max) {
        S = 30.f * (theta - t.theta_max) + t.y[9];
        dS = 30.f;
    } else {
        const float pos = (theta - t.theta_min) * t.inv_h;
        int k = min(8, max(0, (int)floorf(pos)));
        const float B = pos - (float)k;
        const float A = 1.f - B;
        const float yk = t.y[k], yk1 = t.y[k + 1];
        const float mk = t.m[k], mk1 = t.m[k + 1];  // M * h^2 / 6
        S = A * yk + B * yk1 + (A * A * A - A) * mk + (B * B * B - B) * mk1;
        dS = ((yk1 - yk) + (1.f - 3.f * A * A) * mk + (3.f * B * B - 1.f) * mk1) * t.inv_h;
    }
    energy = kk * (S - t.emin);
    const float dE = kk * dS;
    const float uu = norm2(u), vv = norm2(v);
    // dtheta/dx1 = (u x n)/(|u|^2 |n|), dtheta/dx3 = -(v x n)/(|v|^2 |n|)
    const float3 un = make_float3(u.y * n.z - u.z * n.y, u.z * n.x - u.x * n.z, u.x * n.y - u.y * n.x);
    const float3 vn = make_float3(v.y * n.z - v.z * n.y, v.z * n.x - v.x * n.z, v.x * n.y - v.y * n.x);
    const float c1 = -dE / (uu * nlen);
    const float c3 = dE / (vv * nlen);
    f1 = make_float3(c1 * un.x, c1 * un.y, c1 * un.z);
    f3 = make_float3(c3 * vn.x, c3 * vn.y, c3 * vn.z);
}

// Torsion geometry of (x1, x2, x3, x4) from F = x1 - x2, G = x2 - x3,
// H = x4 - x3: cos and sin of the IUPAC dihedral angle (OpenMM's torsion
// convention) without an arc tangent, and the Blondel-Karplus derivatives
// of the angle with respect to the four positions.
struct Torsion {
    float3 A, B;
    float AA, BB, Gl, c, s;
};
__device__ __forceinline__ Torsion torsion_geometry(float3 F, float3 G, float3 H) {
    Torsion t;
    t.A = make_float3(F.y * G.z - F.z * G.y, F.z * G.x - F.x * G.z, F.x * G.y - F.y * G.x);
    t.B = make_float3(H.y * G.z - H.z * G.y, H.z * G.x - H.x * G.z, H.x * G.y - H.y * G.x);
    t.AA = fmaxf(norm2(t.A), 1e-30f);
    t.BB = fmaxf(norm2(t.B), 1e-30f);
    t.Gl = sqrtf(norm2(G));
    const float inv_ab = rsqrtf(t.AA * t.BB);
    t.c = (t.A.x * t.B.x + t.A.y * t.B.y + t.A.z * t.B.z) * inv_ab;
    t.s = -t.Gl * (F.x * t.B.x + F.y * t.B.y + F.z * t.B.z) * inv_ab;
    return t;
}
// Forces f_a = -dE/dphi * dphi/dx_a.
__device__ __forceinline__ void torsion_forces(const Torsion& t, float3 F, float3 G, float3 H,
                                               float dE, float3& f1, float3& f2, float3& f3,
                                               float3& f4) {
    const float3 A = t.A, B = t.B;
    const float ga = t.Gl / t.AA, gb = t.Gl / t.BB;
    const float fg = (F.x * G.x + F.y * G.y + F.z * G.z) / (t.AA * t.Gl);
    const float hg = (H.x * G.x + H.y * G.y + H.z * G.z) / (t.BB * t.Gl);
    // dphi/dx1 = -ga A ; dphi/dx4 = gb B
    const float3 d1 = make_float3(-ga * A.x, -ga * A.y, -ga * A.z);
    const float3 d4 = make_float3(gb * B.x, gb * B.y, gb * B.z);
    // dphi/dx2 = ga A + fg A - hg B ; dphi/dx3 = -gb B - fg A + hg B
    const float3 d2 = make_float3((ga + fg) * A.x - hg * B.x, (ga + fg) * A.y - hg * B.y,
                                  (ga + fg) * A.z - hg * B.z);
    const float3 d3 = make_float3(-fg * A.x + (hg - gb) * B.x, -fg * A.y + (hg - gb) * B.y,
                                  -fg * A.z + (hg - gb) * B.z);
    f1 = make_float3(-dE * d1.x, -dE * d1.y, -dE * d1.z);
    f2 = make_float3(-dE * d2.x, -dE * d2.y, -dE * d2.z);
    f3 = make_float3(-dE * d3.x, -dE * d3.y, -dE * d3.z);
    f4 = make_float3(-dE * d4.x, -dE * d4.y, -dE * d4.z);
}

// Flexible-local dihedral (FlexibleLocalDihedralForceFieldGenerator.cpp:7-59):
// E = k (c - Emin + sum_n a_n cos(n phi) + b_n sin(n phi)), n = 1..3, with
// the multiple angles from cos/sin recurrences.
__device__ __forceinline__ void fld_forces(float3 F, float3 G, float3 H, float kk,
                                           const FldTable& t, float3& f1, float3& f2,
                                           float3& f3, float3& f4, float& energy) {
    const Torsion g = torsion_geometry(F, G, H);
    const float c1 = g.c, s1 = g.s;
    const float c2 = c1 * c1 - s1 * s1, s2 = 2.f * s1 * c1;
    const float c3 = c1 * c2 - s1 * s2, s3 = s1 * c2 + c1 * s2;
    energy = kk * (t.c[0] - t.emin + t.c[1] * c1 + t.c[2] * s1 + t.c[3] * c2 + t.c[4] * s2 +
                   t.c[5] * c3 + t.c[6] * s3);
    const float dE = kk * (-t.c[1] * s1 + t.c[2] * c1 - 2.f * t.c[3] * s2 + 2.f * t.c[4] * c2 -
                           3.f * t.c[5] * s3 + 3.f * t.c[6] * c3);
    torsion_forces(g, F, G, H, dE, f1, f2, f3, f4);
}

// Gaussian dihedral (GaussianDihedralForceFieldGenerator.cpp:5-12):
// E = k exp(-dp^2 / (2 sigma^2)), dp = d - floor((d + pi) / (2 pi)) 2 pi,
// d = phi - theta0; inv2s2 = 1 / (2 sigma^2).
__device__ __forceinline__ void gauss_dihedral_forces(float3 F, float3 G, float3 H, float kk,
                                                      float theta0, float inv2s2, float3& f1,
                                                      float3& f2, float3& f3, float3& f4,
                                                      float& energy) {
    const Torsion g = torsion_geometry(F, G, H);
    const float phi = atan2f(g.s, g.c);
    const float two_pi = 6.2831853071795865f;
    float d = phi - theta0;
    d -= floorf((d + 3.1415926535897932f) * (1.f / two_pi)) * two_pi;
    const float e = kk * expf(-d * d * inv2s2);
    energy = e;
    torsion_forces(g, F, G, H, -2.f * inv2s2 * d * e, f1, f2, f3, f4);
}

// ---------------------------------------------------------------------------
// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw, SC'11),
// written from the published round function.  Box-Muller turns pairs of
// uniforms in (0, 1] into normals.
// ---------------------------------------------------------------------------
struct U4 { uint32_t x, y, z, w; };
__device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int round = 0; round < 10; ++round) {
        const uint32_t lo0 = kPhiloxM0 * c.x;
        const uint32_t hi0 = __umulhi(kPhiloxM0, c.x);
        const uint32_t lo1 = kPhiloxM1 * c.z;
        const uint32_t hi1 = __umulhi(kPhiloxM1, c.z);
        c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        k0 += kPhiloxW0;
        k1 += kPhiloxW1;
    }
    return c;
}
__device__ __forceinline__ float uniform_open0(uint32_t x) {
    return (float)((x >> 8) + 1u) * (1.0f / 16777216.0f);
}
// Three standard normals for (bead, step) of a stream.
__device__ __forceinline__ float3 gaussian3(uint32_t seed, uint32_t stream, uint32_t bead,
                                            unsigned long long step, uint32_t purpose) {
    const U4 r = philox4x32_10(U4{bead, (uint32_t)step, (uint32_t)(step >> 32), purpose}, seed,
                               kPhiloxKey1 ^ stream);
    const float u1 = uniform_open0(r.x), u2 = uniform_open0(r.y);
    const float u3 = uniform_open0(r.z), u4 = uniform_open0(r.w);
    const float a = sqrtf(-2.f * logf(u1));
    const float b = sqrtf(-2.f * logf(u3));
    float s2, c2, s4, c4;
    sincospif(2.f * u2, &s2, &c2);
    sincospif(2.f * u4, &s4, &c4);
    return make_float3(a * c2, a * s2, b * c4);
}

}  // namespace ocm
