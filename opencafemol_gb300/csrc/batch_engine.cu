// batch_engine.cu - persistent shared-memory kernel for many independent
// systems (the batched ensemble and the serving loop).
//
// One CTA per SM (or more, by occupancy) pulls systems from a work queue
// ordered by decreasing cost.  A claimed system is loaded into shared
// memory (float-float positions, parameters, velocities) and advanced for
// the whole chunk without touching global memory except for its neighbour
// list entries beyond the shared-memory share and L2-resident parameters.
// Per MD step:
//   list:     Verlet lists with a 0.3 nm skin, rebuilt when a bead has
//             moved more than half the skin (one thread per bead, j order);
//   forces:   pair units (a bead and a j-range of its list) write the
//             bead's pair force; one lane per chain position evaluates the
//             chain-local bonded terms starting there and the lanes combine
//             them by shuffles; other bonded terms are gathered by each of
//             their beads;
//   update:   Langevin step per bead from the summed forces, bounding boxes,
//             displacement and blow-up checks.
// No atomics on forces: every bead's force is a sum in a fixed order, so a
// system gives the same trajectory alone, in any mix, for any chunking and
// for any threads per CTA.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <tuple>
#include <vector>

#include "batch_engine.hpp"
#include "device_math.cuh"

namespace ocm {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kMaxClusters = 64;  // 2048 beads per system
// Pair work of a bead is split over S adjacent lanes (S = 1, 2, 4 or 8, the
// largest with n * S <= kSplitUnits); sub-lane s sums the list entries whose
// j lies in [s*n/S, (s+1)*n/S).  S depends on n alone, so the FP32 sums, and
// the results, do not depend on the threads per CTA (a CTA with fewer
// threads walks the units in more passes).
constexpr int kSplitUnits = 512;
constexpr int kMaxUnits = kSplitUnits;
constexpr int kMaxSplit = 8;
// Beads are ordered by their longest sub-list at every list build (bucket
// sort over this many buckets), so the 32 lanes of a pair pass carry work of
// similar length.
constexpr int kSortBuckets = 64;
// Shared memory of a system: bytes per bead (state, lists' counts, order)
// and the part that does not grow with the bead count (cluster boxes and
// carries, pair-split offsets, sort buckets, alignment).
constexpr int kBeadBytes = 100;
constexpr int kBeadBytesGeneral = 120;  // with per-bead LJ attraction parameters and labels
constexpr size_t kFixedBytes = (size_t)(32 + 36) * kMaxClusters + 16 + 2 * kMaxUnits + 4 * kSortBuckets;
// A force component beyond this (kJ/mol/nm) marks a blown-up system: far
// above any physical coarse-grained force, and the bound of the plain
// engine's fixed-point accumulators.
constexpr float kForceLimit = 1.0e9f;

__host__ __device__ __forceinline__ int pair_split(int n) {
    int S = 1;
    while (S < kMaxSplit && n * S * 2 <= kSplitUnits) S <<= 1;
    return S;
}

struct BatchArgs {
    BatchSys* sys;
    const int32_t* order;
    const int32_t* order_k;      // steps of each claimed system this launch, or null: k for all
    int n_order;
    int* head;
    double *x, *y, *z;
    float *vx, *vy, *vz;
    const unsigned char* blob;
    int k;
    int nmax;
    double* energy;              // [slot][kNumSlots]
    float* forces;               // eval output [3][nmax]
    uint16_t* lists;             // neighbour-list arena
    uint32_t slots_enabled;
    size_t smem_bytes;           // dynamic shared memory of the launch
    int split_beads;             // a CTA splits into two groups at systems of at most this many beads (0: never)
    int split_bead_bytes;        // host side: shared-memory state bytes per bead (caps split_beads)
};

// Named barrier `bar` over nthreads threads (bar 0 over the whole CTA is
// __syncthreads).
__device__ __forceinline__ void bar_sync(int bar, int nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(nthreads) : "memory");
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

__device__ __forceinline__ float3 lo3(const float* sxl, int nmax, int i) {
    return make_float3(sxl[i], sxl[nmax + i], sxl[2 * nmax + i]);
}

// x_j - x_i of float-float positions, rounded once to FP32.
__device__ __forceinline__ float3 ffsep(const float4* sx, const float* sxl, int nmax, int i, int j) {
    float3 dh, dl;
    ff_sep(sx[i], lo3(sxl, nmax, i), sx[j], lo3(sxl, nmax, j), dh, dl);
    return make_float3(dh.x + dl.x, dh.y + dl.y, dh.z + dl.z);
}

// (hi, lo) += d, renormalised so hi is the FP32 rounding of the sum.
__device__ __forceinline__ void ff_add(float& hi, float& lo, float d) {
    float e;
    const float s = two_sum(hi, d, e);
    const float l = __fadd_rn(lo, e);
    const float h = __fadd_rn(s, l);
    lo = __fsub_rn(l, __fsub_rn(h, s));
    hi = h;
}

__device__ __forceinline__ void add3(float3& a, float3 b) {
    a.x += b.x;
    a.y += b.y;
    a.z += b.z;
}
__device__ __forceinline__ float3 neg3(float3 a) { return make_float3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float3 shfl_up3(float3 v, int d) {
    return make_float3(__shfl_up_sync(kFull, v.x, d), __shfl_up_sync(kFull, v.y, d), __shfl_up_sync(kFull, v.z, d));
}
__device__ __forceinline__ float3 shfl3(float3 v, int src) {
    return make_float3(__shfl_sync(kFull, v.x, src), __shfl_sync(kFull, v.y, src), __shfl_sync(kFull, v.z, src));
}

// Per-term energy accumulators: FP64 sums of the FP32 per-term energies.
struct EnergyAcc {
    double e[kNumSlots];
    __device__ void zero() {
#pragma unroll
        for (int k = 0; k < kNumSlots; ++k) e[k] = 0.0;
    }
};

// ---------------------------------------------------------------------------
// Bonded records as staged in shared memory.
// ---------------------------------------------------------------------------
struct Bonded {
    const float4* bpar;     // bond (p0, p1, r0sq_hi, r0sq_lo)
    const uint32_t* bij;    // i | j << 16 | kind << 30
    const uint2* aij;       // (i | j << 16, k | table << 16)
    const float* ak;
    const uint4* drec;      // (i | j << 16 | gauss << 31, k | l << 16, table / gauss index, k bits)
    const float2* gdp;      // Gaussian dihedral (theta0, 1 / (2 sigma^2))
    const FlaTable* fla;
    const FldTable* fld;
    const uint16_t* cb;     // chain bonds starting at bead b: [cb[b], cb[b+1])
    const uint16_t* ca;     // chain angles
    const uint16_t* cd;     // chain dihedrals
    const uint16_t* gs;     // gather entries of bead b: [gs[b], gs[b+1])
    const uint32_t* gl;     // type << 30 | role << 28 | term index
};

// Bond b: force on its first bead (the second gets the negation), energy.
__device__ __forceinline__ float3 bond_force(const Bonded& B, int b, const float4* sx, const float* sxl, int ns,
                                             float& en, int& slot) {
    const uint32_t ij = B.bij[b];
    const int kind = (int)(ij >> 30);
    slot = bond_slot(kind);
    const int bi = ij & 0xFFFF, bj = (ij >> 16) & 0x3FFF;
    const float4 bp = B.bpar[b];
    float3 dh, dl;
    ff_sep(sx[bi], lo3(sxl, ns, bi), sx[bj], lo3(sxl, ns, bj), dh, dl);
    const float3 d = make_float3(dh.x + dl.x, dh.y + dl.y, dh.z + dl.z);
    const float delta = ff_bond_delta(dh, dl, bp.z, bp.w);
    const float sc = bond_scalar(kind, norm2(d), delta, bp.x, bp.y, bp.z, en);
    return make_float3(-sc * d.x, -sc * d.y, -sc * d.z);
}

// Angle a: forces on its first (f1) and last (f3) bead; the middle one
// gets -(f1 + f3).
__device__ __forceinline__ void angle_force(const Bonded& B, int a, const float4* sx, const float* sxl, int ns,
                                            float3& f1, float3& f3, float& en) {
    const uint2 g = B.aij[a];
    const int gi = g.x & 0xFFFF, gj = g.x >> 16, gk = g.y & 0xFFFF;
    const float3 u = ffsep(sx, sxl, ns, gj, gi);
    const float3 v = ffsep(sx, sxl, ns, gj, gk);
    fla_forces(u, v, B.ak[a], B.fla[g.y >> 16], f1, f3, en);
}

// Dihedral q: forces on its four beads, energy and slot.
__device__ __forceinline__ void dihedral_force(const Bonded& B, int q, const float4* sx, const float* sxl, int ns,
                                               float3& f1, float3& f2, float3& f3, float3& f4, float& en,
                                               int& slot) {
    const uint4 qd = B.drec[q];
    const bool gauss = (qd.x >> 31) != 0;
    slot = gauss ? kSlotGD : kSlotFLD;
    const int qi = qd.x & 0xFFFF, qj = (qd.x >> 16) & 0x7FFF, qk = qd.y & 0xFFFF, ql = qd.y >> 16;
    const float3 F = ffsep(sx, sxl, ns, qj, qi);
    const float3 G = ffsep(sx, sxl, ns, qk, qj);
    const float3 H = ffsep(sx, sxl, ns, qk, ql);
    if (gauss) {
        const float2 gp = B.gdp[qd.z];
        gauss_dihedral_forces(F, G, H, __uint_as_float(qd.w), gp.x, gp.y, f1, f2, f3, f4, en);
    } else {
        fld_forces(F, G, H, __uint_as_float(qd.w), B.fld[qd.z], f1, f2, f3, f4, en);
    }
}

__device__ __forceinline__ bool slot_on(uint32_t slots_en, int slot) { return (slots_en >> slot) & 1u; }

// Bonded force on bead b = I * 32 + lane of cluster I (one warp).  The lane
// evaluates every chain-local term starting at b (bonds b-b+1, angles
// b..b+2, dihedrals b..b+3) once, keeping its contributions to b..b+3; the
// lanes then add what lanes 1..3 below them send up, in a fixed order, and
// the three contributions that cross into cluster I + 1 go to carry[I].
// Terms that are not chain-local are evaluated by each of their beads
// (gather entries) and only that bead's share is kept.
template <bool ENERGY>
__device__ __forceinline__ float3 bonded_cluster(const Bonded& B, int I, int n, int lane, const float4* sx,
                                                 const float* sxl, int ns, uint32_t slots_en, float3* carry,
                                                 EnergyAcc& ea) {
    const int b = I * 32 + lane;
    float3 o0 = make_float3(0.f, 0.f, 0.f), o1 = o0, o2 = o0, o3 = o0;
    if (b < n) {
        for (int t = B.cb[b]; t < B.cb[b + 1]; ++t) {
            float en;
            int sl;
            const float3 f = bond_force(B, t, sx, sxl, ns, en, sl);
            if (!slot_on(slots_en, sl)) continue;
            add3(o0, f);
            add3(o1, neg3(f));
            if (ENERGY) ea.e[sl] += (double)en;
        }
        if (slot_on(slots_en, kSlotFLA))
            for (int t = B.ca[b]; t < B.ca[b + 1]; ++t) {
                float3 f1, f3;
                float en;
                angle_force(B, t, sx, sxl, ns, f1, f3, en);
                add3(o0, f1);
                add3(o2, f3);
                add3(o1, make_float3(-f1.x - f3.x, -f1.y - f3.y, -f1.z - f3.z));
                if (ENERGY) ea.e[kSlotFLA] += (double)en;
            }
        for (int t = B.cd[b]; t < B.cd[b + 1]; ++t) {
            float3 f1, f2, f3, f4;
            float en;
            int sl;
            dihedral_force(B, t, sx, sxl, ns, f1, f2, f3, f4, en, sl);
            if (!slot_on(slots_en, sl)) continue;
            add3(o0, f1);
            add3(o1, f2);
            add3(o2, f3);
            add3(o3, f4);
            if (ENERGY) ea.e[sl] += (double)en;
        }
    }
    // contributions of the three chain positions below, in the order
    // 1, 2, 3 positions back
    const float3 u1 = shfl_up3(o1, 1), u2 = shfl_up3(o2, 2), u3 = shfl_up3(o3, 3);
    float3 fb = o0;
    if (lane >= 1) add3(fb, u1);
    if (lane >= 2) add3(fb, u2);
    if (lane >= 3) add3(fb, u3);
    // what lanes 29..31 send into the next cluster's first three beads
    const float3 a1 = shfl3(o1, 31), a2 = shfl3(o2, 30), a3 = shfl3(o3, 29);
    const float3 b2 = shfl3(o2, 31), b3 = shfl3(o3, 30);
    const float3 c3 = shfl3(o3, 31);
    if (lane == 0) {
        float3 c0 = a1;
        add3(c0, a2);
        add3(c0, a3);
        float3 c1 = b2;
        add3(c1, b3);
        carry[3 * I] = c0;
        carry[3 * I + 1] = c1;
        carry[3 * I + 2] = c3;
    }
    if (b < n) {
        for (int g = B.gs[b]; g < B.gs[b + 1]; ++g) {
            const uint32_t e = B.gl[g];
            const int type = (int)(e >> 30), role = (int)((e >> 28) & 3u), t = (int)(e & 0x0FFFFFFFu);
            float en;
            float3 f;
            int sl;
            if (type == 0) {
                f = bond_force(B, t, sx, sxl, ns, en, sl);
                if (role == 1) f = neg3(f);
            } else if (type == 1) {
                sl = kSlotFLA;
                float3 f1, f3;
                angle_force(B, t, sx, sxl, ns, f1, f3, en);
                f = role == 0 ? f1 : role == 2 ? f3 : make_float3(-f1.x - f3.x, -f1.y - f3.y, -f1.z - f3.z);
            } else {
                float3 f1, f2, f3, f4;
                dihedral_force(B, t, sx, sxl, ns, f1, f2, f3, f4, en, sl);
                f = role == 0 ? f1 : role == 1 ? f2 : role == 2 ? f3 : f4;
            }
            if (!slot_on(slots_en, sl)) continue;
            add3(fb, f);
            if (ENERGY && role == 0) ea.e[sl] += (double)en;
        }
    }
    return fb;
}

// Bounding box of cluster I from the FP32 positions (warp-wide).
__device__ __forceinline__ void cluster_bbox(int I, int n, const float4* sx, float4* bc,
                                             float4* bh, int lane) {
    const int b = I * 32 + lane;
    const float4 base = sx[I * 32];
    float3 d = make_float3(0.f, 0.f, 0.f);
    if (b < n) {
        const float4 p = sx[b];
        d = make_float3(p.x - base.x, p.y - base.y, p.z - base.z);
    }
    float lx = d.x, ly = d.y, lz = d.z, hx = d.x, hy = d.y, hz = d.z;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lx = fminf(lx, __shfl_xor_sync(kFull, lx, o));
        ly = fminf(ly, __shfl_xor_sync(kFull, ly, o));
        lz = fminf(lz, __shfl_xor_sync(kFull, lz, o));
        hx = fmaxf(hx, __shfl_xor_sync(kFull, hx, o));
        hy = fmaxf(hy, __shfl_xor_sync(kFull, hy, o));
        hz = fmaxf(hz, __shfl_xor_sync(kFull, hz, o));
    }
    if (lane == 0) {
        bc[I] = make_float4(base.x + 0.5f * (lx + hx), base.y + 0.5f * (ly + hy),
                            base.z + 0.5f * (lz + hz), 0.f);
        bh[I] = make_float4(0.5f * (hx - lx), 0.5f * (hy - ly), 0.5f * (hz - lz), 0.f);
    }
}

// Exclusion bits of (i, j) for the j of an increasing walk: ep / ej track
// the position in bead i's exclusion row (j | bits << 24, j increasing).
__device__ __forceinline__ uint32_t excl_walk(int j, int& ep, int& ej, int e1, const int32_t* __restrict__ ex) {
    while (ej < j) {
        ++ep;
        ej = ep < e1 ? (ex[ep] & 0xFFFFFF) : 0x7FFFFFFF;
    }
    return ej == j ? ((uint32_t)ex[ep] >> 24) : 0u;
}

template <bool LABELS>
__device__ __forceinline__ uint32_t label_bits(uint32_t labi, uint32_t labj, const PairConsts& pc) {
    uint32_t bits = 0u;
    if (LABELS) {
#pragma unroll
        for (int term = 0; term < 4; ++term)
            if ((pc.uses_labels & (1 << term)) && !labels_allow(labi, labj, term, pc.allow[term]))
                bits |= 1u << term;
    }
    return bits;
}

// Neighbour list of every bead of the claimed system, built by one thread
// per bead: all j != i whose FP32 r^2 (canonical form) is below cut2, in
// increasing j, so the list and every FP32 sum over it are deterministic.
// Entry = j | (excluded-term bits << 11); pairs excluded for every present
// term are dropped.  Entry k of bead i lives in shared memory at
// slist[k * npad + i] for k < cap_s and in global memory at
// glist[k * npad + i] for cap_s <= k < maxn.  Sets *overflow when a list
// exceeds maxn.  Then bord = the beads in decreasing length of their
// longest sub-list (bucket sort; ties in any order), through the group's
// barrier `bar`; tmp (n words) and hist (kSortBuckets words, zero on entry
// and on return) are scratch.
template <bool LABELS>
__device__ __forceinline__ void build_lists(int n, int nt, int npad, int maxn, int cap_s, float cut2,
                                            const float4* sx, const uint32_t* slab,
                                            const float4* bc, const float4* bh,
                                            const int32_t* __restrict__ ex_start,
                                            const int32_t* __restrict__ ex,
                                            const PairConsts& pc, uint16_t* slist,
                                            uint16_t* __restrict__ glist, uint16_t* scnt,
                                            float* sref, int nmax, int tid, int threads,
                                            int S, uint16_t* sseg, int* overflow, uint16_t* bord,
                                            int* hist, uint32_t* tmp, int bar) {
    const float3 nobox = make_float3(0.f, 0.f, 0.f);
    const uint32_t present = (uint32_t)pc.terms;
    for (int i = tid; i < n; i += threads) {
        const float4 xi = sx[i];
        const uint32_t labi = LABELS ? slab[i] : 0u;
        int cnt = 0;
        int seg0 = 0, longest = 0;  // start of the current sub-list, longest so far
        // list offset where each j-range of the pair split starts
        int s_next = 1;
        int jb = S > 1 ? n / S : 0x7FFFFFFF;
        if (S > 1) sseg[i * S] = 0;
        int ep = ex_start[i];
        const int e1 = ex_start[i + 1];
        int ej = ep < e1 ? (ex[ep] & 0xFFFFFF) : 0x7FFFFFFF;
        for (int J = 0; J < nt; ++J) {
            const float4 c = bc[J], h = bh[J];
            const float gx = fmaxf(0.f, fabsf(xi.x - c.x) - h.x);
            const float gy = fmaxf(0.f, fabsf(xi.y - c.y) - h.y);
            const float gz = fmaxf(0.f, fabsf(xi.z - c.z) - h.z);
            if (gx * gx + gy * gy + gz * gz >= cut2) continue;
            const int j1 = min(n, J * 32 + 32);
            for (int j = J * 32; j < j1; ++j) {
                if (j == i) continue;
                const float r2 = norm2(separation<false>(xi, sx[j], nobox, nobox));
                if (!(r2 < cut2)) continue;
                uint32_t bits = excl_walk(j, ep, ej, e1, ex);
                if (LABELS) bits |= label_bits<true>(labi, slab[j], pc);
                if ((bits & present) == present) continue;
                while (j >= jb) {
                    const int c = min(cnt, maxn);
                    longest = max(longest, c - seg0);
                    seg0 = c;
                    sseg[i * S + s_next] = (uint16_t)c;
                    ++s_next;
                    jb = s_next < S ? (s_next * n) / S : 0x7FFFFFFF;
                }
                const uint16_t e = (uint16_t)(j | (bits << 11));
                if (cnt < cap_s) slist[cnt * npad + i] = e;
                else if (cnt < maxn) glist[(size_t)cnt * npad + i] = e;
                ++cnt;
            }
        }
        if (cnt > maxn) {
            atomicOr(overflow, 1);
            cnt = maxn;
        }
        for (; s_next < S; ++s_next) sseg[i * S + s_next] = (uint16_t)cnt;
        scnt[i] = (uint16_t)cnt;
        sref[i] = xi.x;
        sref[nmax + i] = xi.y;
        sref[2 * nmax + i] = xi.z;
        longest = max(longest, cnt - seg0);
        const int bucket = longest < 32 ? longest : min(kSortBuckets - 1, 32 + ((longest - 32) >> 2));
        tmp[i] = (uint32_t)bucket | (uint32_t)atomicAdd(&hist[bucket], 1) << 8;
    }
    bar_sync(bar, threads);
    if (tid < 32) {
        // exclusive offsets, buckets in decreasing order: lane l holds
        // buckets 63 - 2l and 62 - 2l
        const int h0 = hist[kSortBuckets - 1 - 2 * tid], h1 = hist[kSortBuckets - 2 - 2 * tid];
        const int pair = h0 + h1;
        int incl = pair;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(kFull, incl, o);
            if (tid >= o) incl += v;
        }
        hist[kSortBuckets - 1 - 2 * tid] = incl - pair;
        hist[kSortBuckets - 2 - 2 * tid] = incl - pair + h0;
    }
    bar_sync(bar, threads);
    for (int i = tid; i < n; i += threads) {
        const uint32_t t = tmp[i];
        bord[hist[t & 255u] + (int)(t >> 8)] = (uint16_t)i;
    }
    bar_sync(bar, threads);
    if (tid < kSortBuckets) hist[tid] = 0;
}

template <int TERMS, bool ENERGY>
__device__ __forceinline__ void pair_accumulate(int i, int j, float4 xi, float4 xj, float4 p0i, float4 p1i,
                                                const float4* sp0, const float4* sp1, uint32_t bits,
                                                const PairConsts& pc, float3& fa, EnergyAcc& ea) {
    const float3 nobox = make_float3(0.f, 0.f, 0.f);
    const float3 d = separation<false>(xi, xj, nobox, nobox);
    const float r2 = norm2(d);
    if (r2 < pc.list_rc2) {
        const float4 p0j = sp0[j];
        const float4 p1j = (TERMS & kTermLJA) ? sp1[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        PairEnergy e;
        e.zero();
        const float s = pair_scalar<TERMS, ENERGY>(r2, p0i, p0j, p1i, p1j, bits, pc, e);
        fa.x -= s * d.x;
        fa.y -= s * d.y;
        fa.z -= s * d.z;
        if (ENERGY) {
            // every pair is met from both of its beads
            ea.e[kSlotEXV] += 0.5 * (double)e.exv;
            ea.e[kSlotDH] += 0.5 * (double)e.dh;
            ea.e[kSlotLJR] += 0.5 * (double)e.ljr;
            ea.e[kSlotLJA] += 0.5 * (double)e.lja;
        }
    }
}

// Pair forces of list entries [k0, k1) of bead i in one memory space,
// four entries per iteration: the entries' loads are issued first, and the
// cutoff test selects the result instead of branching, so the four pair
// evaluations interleave.  One accumulator in list (= increasing j) order:
// entries outside the cutoff contribute exactly zero.
template <int TERMS, bool ENERGY>
__device__ __forceinline__ void list_range(int i, int k0, int k1, int npad, const uint16_t* __restrict__ L,
                                           float4 xi, float4 p0i, float4 p1i, const float4* sx,
                                           const float4* sp0, const float4* sp1, uint32_t excl_all,
                                           const PairConsts& pc, float3& fa, EnergyAcc& ea) {
    const float3 nobox = make_float3(0.f, 0.f, 0.f);
    for (int k = k0; k < k1; k += 4) {
        uint32_t ent[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) ent[u] = k + u < k1 ? (uint32_t)L[(size_t)(k + u) * npad + i] : (uint32_t)i;
        float4 xj[4], p0j[4], p1j[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int j = (int)(ent[u] & 2047u);
            xj[u] = sx[j];
            p0j[u] = sp0[j];
            p1j[u] = (TERMS & kTermLJA) ? sp1[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const float3 d = separation<false>(xi, xj[u], nobox, nobox);
            const float r2 = norm2(d);
            const bool in = k + u < k1 && r2 < pc.list_rc2;
            PairEnergy e;
            e.zero();
            float sc = pair_scalar<TERMS, ENERGY>(in ? r2 : pc.list_rc2, p0i, p0j[u], p1i, p1j[u],
                                                  (ent[u] >> 11) | excl_all, pc, e);
            sc = in ? sc : 0.f;
            fa.x -= sc * d.x;
            fa.y -= sc * d.y;
            fa.z -= sc * d.z;
            if (ENERGY && in) {
                // every pair is met from both of its beads
                ea.e[kSlotEXV] += 0.5 * (double)e.exv;
                ea.e[kSlotDH] += 0.5 * (double)e.dh;
                ea.e[kSlotLJR] += 0.5 * (double)e.ljr;
                ea.e[kSlotLJA] += 0.5 * (double)e.lja;
            }
        }
    }
}

// Pair forces on bead i from list entries [k0, k1): the shared-memory part
// (k < cap_s), then the part in global memory.
template <int TERMS, bool ENERGY>
__device__ __forceinline__ float3 list_forces(int i, int k0, int k1, int cap_s, int npad,
                                              const uint16_t* slist,
                                              const uint16_t* __restrict__ glist,
                                              const float4* sx, const float4* sp0,
                                              const float4* sp1, uint32_t excl_all,
                                              const PairConsts& pc, EnergyAcc& ea) {
    const float4 xi = sx[i];
    const float4 p0i = sp0[i];
    const float4 p1i = (TERMS & kTermLJA) ? sp1[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    float3 fa = make_float3(0.f, 0.f, 0.f);
    const int ks = min(k1, cap_s);
    if (k0 < ks) list_range<TERMS, ENERGY>(i, k0, ks, npad, slist, xi, p0i, p1i, sx, sp0, sp1, excl_all, pc, fa, ea);
    const int kg = max(k0, cap_s);
    if (kg < k1) list_range<TERMS, ENERGY>(i, kg, k1, npad, glist, xi, p0i, p1i, sx, sp0, sp1, excl_all, pc, fa, ea);
    return fa;
}

// The same sum without a list, for a system whose list overflowed: every
// j in [j0, j1) in increasing order, the clusters culled by their bounding
// boxes at the cutoff.  The nonzero contributions and their order are those
// of the list walk, so the force is bit-identical to it.
template <int TERMS, bool LABELS, bool ENERGY>
__device__ __forceinline__ float3 scan_forces(int i, int j0, int j1, int nt, const float4* sx, const float4* sp0,
                                              const float4* sp1, const uint32_t* slab, const float4* bc,
                                              const float4* bh, float cull2, const int32_t* __restrict__ ex_start,
                                              const int32_t* __restrict__ ex, uint32_t excl_all,
                                              const PairConsts& pc, EnergyAcc& ea) {
    const float4 xi = sx[i];
    const float4 p0i = sp0[i];
    const float4 p1i = (TERMS & kTermLJA) ? sp1[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const uint32_t labi = LABELS ? slab[i] : 0u;
    const uint32_t present = (uint32_t)pc.terms;
    int ep = ex_start[i];
    const int e1 = ex_start[i + 1];
    int ej = ep < e1 ? (ex[ep] & 0xFFFFFF) : 0x7FFFFFFF;
    float3 fa = make_float3(0.f, 0.f, 0.f);
    for (int J = j0 >> 5; J < nt && J * 32 < j1; ++J) {
        const float4 c = bc[J], h = bh[J];
        const float gx = fmaxf(0.f, fabsf(xi.x - c.x) - h.x);
        const float gy = fmaxf(0.f, fabsf(xi.y - c.y) - h.y);
        const float gz = fmaxf(0.f, fabsf(xi.z - c.z) - h.z);
        if (gx * gx + gy * gy + gz * gz >= cull2) continue;
        const int ja = max(j0, J * 32), jz = min(j1, J * 32 + 32);
        for (int j = ja; j < jz; ++j) {
            if (j == i) continue;
            uint32_t bits = excl_walk(j, ep, ej, e1, ex);
            if (LABELS) bits |= label_bits<true>(labi, slab[j], pc);
            if ((bits & present) == present) continue;
            pair_accumulate<TERMS, ENERGY>(i, j, xi, sx[j], p0i, p1i, sp0, sp1, bits | excl_all, pc, fa, ea);
        }
    }
    return fa;
}

// One claimed system (order entry q, slot `slot`) advanced by a group of GT
// threads (gtid = 0..GT-1) whose barrier is `bar` (0: the whole CTA), in
// the group's shared memory [gsmem, gsmem + gsmem_bytes), with the group's
// shared words (s_move[2], s_overflow, s_bad, s_energy[kNumSlots]).
template <int GT, int TERMS, bool LABELS, bool ENERGY, bool INTEGRATE>
__device__ __forceinline__ void run_system(const BatchArgs& a, int q, int slot, int gtid, int bar,
                                           unsigned char* gsmem, size_t gsmem_bytes, int* s_move,
                                           int* s_overflow, int* s_bad, double* s_energy, int* s_item) {
    constexpr int NWG = GT / 32;
    constexpr int BPT = (32 * kMaxClusters + GT - 1) / GT;  // cluster rows per warp in the update
    const int lane = gtid & 31, gwarp = gtid >> 5;
    const int nmax = a.nmax;  // stride of the global force output
    const float nan = __int_as_float(0x7fc00000);
    const BatchSys& R = a.sys[slot];
    const int n = R.n, nt = R.nt, npad = nt * 32;
    const PairConsts pc = R.pc;
    const LangevinConsts lc = R.lc;
    const long long boff = R.bead_off;
    const unsigned char* blob = a.blob + R.blob_off;
    const float4* gp0 = reinterpret_cast<const float4*>(blob + R.off_p0);
    const float4* gp1 = reinterpret_cast<const float4*>(blob + R.off_p1);
    const uint32_t* glab = reinterpret_cast<const uint32_t*>(blob + R.off_lab);
    const float* ginvm = reinterpret_cast<const float*>(blob + R.off_invm);
    // ---- shared-memory layout of this system, arrays of stride ns ----
    // Positions are float-float: hi parts in sx (pair arithmetic), lo
    // parts in sxl; x = hi + lo carries ~48 significant bits.  fp / fb:
    // each bead's pair and bonded force of the current step.
    const int ns = npad;
    float* fp = reinterpret_cast<float*>(gsmem);
    float* fb = reinterpret_cast<float*>(gsmem + 12 * (size_t)ns);
    float4* sx = reinterpret_cast<float4*>(gsmem + 24 * (size_t)ns);
    float4* sp0 = reinterpret_cast<float4*>(gsmem + 40 * (size_t)ns);
    float* sxl = reinterpret_cast<float*>(gsmem + 56 * (size_t)ns);
    float* sv = reinterpret_cast<float*>(gsmem + 68 * (size_t)ns);
    float* sim = reinterpret_cast<float*>(gsmem + 80 * (size_t)ns);
    float* sref = reinterpret_cast<float*>(gsmem + 84 * (size_t)ns);
    uint16_t* scnt = reinterpret_cast<uint16_t*>(gsmem + 96 * (size_t)ns);
    uint16_t* bord = reinterpret_cast<uint16_t*>(gsmem + 98 * (size_t)ns);
    size_t off = (size_t)kBeadBytes * ns;
    float4* sp1 = nullptr;
    uint32_t* slab = nullptr;
    if ((TERMS & kTermLJA) || LABELS) {
        sp1 = reinterpret_cast<float4*>(gsmem + off);
        slab = reinterpret_cast<uint32_t*>(gsmem + off + 16 * (size_t)ns);
        off += 20 * (size_t)ns;
    }
    float4* bc = reinterpret_cast<float4*>(gsmem + off);
    float4* bh = bc + nt;
    off += 32 * (size_t)nt;
    float3* carry = reinterpret_cast<float3*>(gsmem + off);
    off += 36 * (size_t)nt;
    off = (off + 15) & ~(size_t)15;
    uint16_t* sseg = reinterpret_cast<uint16_t*>(gsmem + off);
    off += 2 * kMaxUnits;
    int* hist = reinterpret_cast<int*>(gsmem + off);
    off += 4 * kSortBuckets;
    // bonded records and tables: staged in shared memory when they fit,
    // read from the blob otherwise
    const unsigned char* gbonded = blob + R.off_bonded;
    const bool bonded_smem = off + (size_t)R.bonded_bytes <= gsmem_bytes;
    unsigned char* sbonded = gsmem + off;
    if (bonded_smem) off += (size_t)R.bonded_bytes;
    const unsigned char* bsrc = bonded_smem ? sbonded : gbonded;
    Bonded B;
    B.bpar = reinterpret_cast<const float4*>(bsrc + R.rb_p);
    B.bij = reinterpret_cast<const uint32_t*>(bsrc + R.rb_ij);
    B.aij = reinterpret_cast<const uint2*>(bsrc + R.ra_ij);
    B.ak = reinterpret_cast<const float*>(bsrc + R.ra_k);
    B.drec = reinterpret_cast<const uint4*>(bsrc + R.rd);
    B.gdp = reinterpret_cast<const float2*>(bsrc + R.rgd);
    B.fla = reinterpret_cast<const FlaTable*>(bsrc + R.rfla);
    B.fld = reinterpret_cast<const FldTable*>(bsrc + R.rfld);
    B.cb = reinterpret_cast<const uint16_t*>(bsrc + R.rcb);
    B.ca = reinterpret_cast<const uint16_t*>(bsrc + R.rca);
    B.cd = reinterpret_cast<const uint16_t*>(bsrc + R.rcd);
    B.gs = reinterpret_cast<const uint16_t*>(bsrc + R.rgs);
    B.gl = reinterpret_cast<const uint32_t*>(bsrc + R.rgl);
    uint16_t* slist = reinterpret_cast<uint16_t*>(gsmem + off);
    const size_t list_bytes = gsmem_bytes > off ? gsmem_bytes - off : 0;
    const int32_t* ex_start = reinterpret_cast<const int32_t*>(blob + R.off_ex_start);
    const int32_t* exl = reinterpret_cast<const int32_t*>(blob + R.off_ex);
    uint16_t* glist = a.lists + R.list_off;
    const int maxn = R.maxn;
    // entries per bead kept in shared memory (multiple of 4)
    const int cap_s = min(maxn, (int)(list_bytes / (2 * (size_t)npad)) & ~3);
    const int S = pair_split(n);
    const unsigned long long step0 = R.steps_done;
    int K = 1;
    if (INTEGRATE) {
        const unsigned long long left = R.steps_target > step0 ? R.steps_target - step0 : 0ull;
        K = (int)min((unsigned long long)(a.order_k ? a.order_k[q] : a.k), left);
    }
    const uint32_t slots_en = INTEGRATE ? 0xffffffffu : a.slots_enabled;
    uint32_t excl_all = 0u;
    if (!(slots_en & (1u << kSlotEXV))) excl_all |= kTermEXV;
    if (!(slots_en & (1u << kSlotDH))) excl_all |= kTermDH;
    if (!(slots_en & (1u << kSlotLJR))) excl_all |= kTermLJR;
    if (!(slots_en & (1u << kSlotLJA))) excl_all |= kTermLJA;
    const bool pairs_on = (pc.terms & ~excl_all) != 0;

    // ---- load ----
    for (int b = gtid; b < npad; b += GT) {
        if (b < n) {
            const double px = a.x[boff + b], py = a.y[boff + b], pz = a.z[boff + b];
            const float hx = __double2float_rn(px), hy = __double2float_rn(py),
                        hz = __double2float_rn(pz);
            sx[b] = make_float4(hx, hy, hz, 0.f);
            sxl[b] = __double2float_rn(px - (double)hx);
            sxl[ns + b] = __double2float_rn(py - (double)hy);
            sxl[2 * ns + b] = __double2float_rn(pz - (double)hz);
            sp0[b] = gp0[b];
            sv[b] = a.vx[boff + b];
            sv[ns + b] = a.vy[boff + b];
            sv[2 * ns + b] = a.vz[boff + b];
            sim[b] = ginvm[b];
            if ((TERMS & kTermLJA) || LABELS) {
                sp1[b] = gp1[b];
                slab[b] = glab[b];
            }
        } else {
            sx[b] = make_float4(nan, nan, nan, 0.f);
            sp0[b] = make_float4(0.f, 0.f, 0.f, 0.f);
            sim[b] = 0.f;
            if ((TERMS & kTermLJA) || LABELS) {
                sp1[b] = make_float4(0.f, 0.f, 0.f, 0.f);
                slab[b] = 0xffffffffu;
            }
        }
    }
    if (bonded_smem) {
        const uint4* src = reinterpret_cast<const uint4*>(gbonded);
        uint4* dst = reinterpret_cast<uint4*>(sbonded);
        for (int q = gtid; q < R.bonded_bytes / 16; q += GT) dst[q] = src[q];
    }
    for (int k = gtid; k < kSortBuckets; k += GT) hist[k] = 0;
    for (int b = gtid; b < n; b += GT) bord[b] = (uint16_t)b;  // until the first list build
    if (gtid == 0) *s_item = 0;
    bar_sync(bar, GT);
    for (int I = gwarp; I < nt; I += NWG) cluster_bbox(I, n, sx, bc, bh, lane);
    bar_sync(bar, GT);

    // list cutoff = largest pair cutoff + skin; the scan culls at the
    // cutoff (with a margin for the FP32 box arithmetic)
    const float rc = sqrtf(pc.list_rc2);
    const float lcut = (rc + R.skin) * 1.0001f;
    const float lcut2 = lcut * lcut;
    const float tcut = rc * 1.0001f + 1e-4f;
    const float tcut2 = tcut * tcut;
    const float half_skin2 = 0.25f * R.skin * R.skin;
    bool use_scan = false;
    bool need_build = pairs_on;
    int builds = 0;
    int st_done = 0;
    EnergyAcc ea;
    if (ENERGY) ea.zero();

    for (int st = 0; st < K; ++st) {
        if (need_build && !use_scan) {
            // fb is free until the bonded terms of this step: sort scratch
            build_lists<LABELS>(n, nt, npad, maxn, cap_s, lcut2, sx, slab, bc, bh, ex_start, exl,
                                pc, slist, glist, scnt, sref, ns, gtid, GT, S, sseg,
                                s_overflow, bord, hist, reinterpret_cast<uint32_t*>(fb), bar);
            ++builds;
            bar_sync(bar, GT);
            use_scan = *s_overflow != 0;
        }
        const unsigned long long step = step0 + (unsigned long long)st;
        // ---- forces: warps claim work items from the group's counter,
        // the bonded clusters first, then the pair passes, longest first
        // (claiming the longest passes before the bonded clusters measured
        // slower).  Pair pass p covers units u = 32 p + lane
        // of the sorted beads: the S units of bead bord[u / S] are adjacent
        // lanes (sub-lane u % S sums the list entries whose j lies in its
        // j-range); their partial sums meet in a fixed butterfly and the
        // first sub-lane stores the bead's pair force.  Every bead's sum is
        // the same whichever warp and lanes compute it. ----
        const int n_pass = pairs_on ? (n * S + 31) >> 5 : 0;
        const int lg_s = __ffs(S) - 1;
        while (true) {
            int it = 0;
            if (lane == 0) it = atomicAdd(s_item, 1);
            it = __shfl_sync(kFull, it, 0);
            if (it >= nt + n_pass) break;
            if (it < nt) {
                const float3 f = bonded_cluster<ENERGY>(B, it, n, lane, sx, sxl, ns, slots_en, carry, ea);
                const int b = it * 32 + lane;
                if (b < n) {
                    fb[b] = f.x;
                    fb[ns + b] = f.y;
                    fb[2 * ns + b] = f.z;
                }
                continue;
            }
            const int u = ((it - nt) << 5) + lane;
            const int sb = u >> lg_s, sr = u & (S - 1);
            const int i = sb < n ? (int)bord[sb] : n;
            float3 fi = make_float3(0.f, 0.f, 0.f);
            if (i < n) {
                if (!use_scan) {
                    const int k0 = S > 1 ? (int)sseg[i * S + sr] : 0;
                    const int k1 = sr == S - 1 ? (int)scnt[i] : (int)sseg[i * S + sr + 1];
                    fi = list_forces<TERMS, ENERGY>(i, k0, k1, cap_s, npad, slist, glist, sx, sp0, sp1,
                                                    excl_all, pc, ea);
                } else {
                    const int j0 = (sr * n) / S, j1 = sr == S - 1 ? n : ((sr + 1) * n) / S;
                    fi = scan_forces<TERMS, LABELS, ENERGY>(i, j0, j1, nt, sx, sp0, sp1, slab, bc, bh,
                                                            tcut2, ex_start, exl, excl_all, pc, ea);
                }
            }
            for (int o = 1; o < S; o <<= 1) {
                fi.x += __shfl_xor_sync(kFull, fi.x, o);
                fi.y += __shfl_xor_sync(kFull, fi.y, o);
                fi.z += __shfl_xor_sync(kFull, fi.z, o);
            }
            if (i < n && sr == 0) {
                fp[i] = fi.x;
                fp[ns + i] = fi.y;
                fp[2 * ns + i] = fi.z;
            }
        }
        bar_sync(bar, GT);
        if (gtid == 0) *s_item = 0;  // read again only after the next barrier
        if (!INTEGRATE) break;
        // ---- Langevin update, bounding boxes, displacement and
        // blow-up checks; bead b = I * 32 + lane of cluster I = gwarp +
        // c * NWG ----
        const int mv = st & 1;
#pragma unroll 4
        for (int c = 0; c < BPT; ++c) {
            const int I = gwarp + c * NWG;
            if (I >= nt) break;
            const int b = I * 32 + lane;
            bool moved = false, bad = false;
            if (b < n) {
                float fx = fb[b], fy = fb[ns + b], fz = fb[2 * ns + b];
                if (pairs_on) {
                    fx = fp[b] + fx;
                    fy = fp[ns + b] + fy;
                    fz = fp[2 * ns + b] + fz;
                }
                if (lane < 3 && I > 0) {
                    const float3 cin = carry[3 * (I - 1) + lane];
                    fx += cin.x;
                    fy += cin.y;
                    fz += cin.z;
                }
                bad = !(fabsf(fx) <= kForceLimit && fabsf(fy) <= kForceLimit && fabsf(fz) <= kForceLimit);
                const float im = sim[b];
                if (im > 0.f) {
                    const float3 g = gaussian3(lc.seed, lc.stream, (uint32_t)b, step, kPurposeLangevin);
                    const float sq = sqrtf(im) * lc.noise;
                    const float fs = lc.fscale * im;
                    const float vx = lc.vscale * sv[b] + fs * fx + sq * g.x;
                    const float vy = lc.vscale * sv[ns + b] + fs * fy + sq * g.y;
                    const float vz = lc.vscale * sv[2 * ns + b] + fs * fz + sq * g.z;
                    sv[b] = vx;
                    sv[ns + b] = vy;
                    sv[2 * ns + b] = vz;
                    float4 h = sx[b];
                    ff_add(h.x, sxl[b], vx * lc.dt);
                    ff_add(h.y, sxl[ns + b], vy * lc.dt);
                    ff_add(h.z, sxl[2 * ns + b], vz * lc.dt);
                    sx[b] = h;
                    bad = bad || !(isfinite(h.x) && isfinite(h.y) && isfinite(h.z));
                    const float dx = h.x - sref[b], dy = h.y - sref[ns + b], dz = h.z - sref[2 * ns + b];
                    moved = dx * dx + dy * dy + dz * dz > half_skin2;
                }
            }
            if (__any_sync(kFull, moved) && lane == 0) atomicOr(&s_move[mv], 1);
            if (__any_sync(kFull, bad) && lane == 0) atomicOr(s_bad, 1);
            __syncwarp();
            cluster_bbox(I, n, sx, bc, bh, lane);
        }
        bar_sync(bar, GT);
        st_done = st + 1;
        if (*s_bad) break;  // the system blew up this step: stop advancing it
        need_build = s_move[mv] != 0;
        if (gtid == 0) s_move[mv ^ 1] = 0;
    }

    // ---- write back ----
    if (INTEGRATE) {
        for (int b = gtid; b < n; b += GT) {
            const float4 h = sx[b];
            a.x[boff + b] = (double)h.x + (double)sxl[b];
            a.y[boff + b] = (double)h.y + (double)sxl[ns + b];
            a.z[boff + b] = (double)h.z + (double)sxl[2 * ns + b];
            a.vx[boff + b] = sv[b];
            a.vy[boff + b] = sv[ns + b];
            a.vz[boff + b] = sv[2 * ns + b];
        }
        if (gtid == 0) {
            a.sys[slot].steps_done = step0 + (unsigned long long)st_done;
            a.sys[slot].builds = builds;
            if (*s_overflow) a.sys[slot].overflow = 1;
            if (*s_bad) a.sys[slot].status = kBatchStatusBlownUp;
        }
    } else {
        bool bad = false;
        for (int b = gtid; b < n; b += GT) {
            float fx = fb[b], fy = fb[ns + b], fz = fb[2 * ns + b];
            if (pairs_on) {
                fx = fp[b] + fx;
                fy = fp[ns + b] + fy;
                fz = fp[2 * ns + b] + fz;
            }
            const int I = b >> 5, l = b & 31;
            if (l < 3 && I > 0) {
                const float3 cin = carry[3 * (I - 1) + l];
                fx += cin.x;
                fy += cin.y;
                fz += cin.z;
            }
            bad = bad || !(fabsf(fx) <= kForceLimit && fabsf(fy) <= kForceLimit && fabsf(fz) <= kForceLimit);
            a.forces[b] = fx;
            a.forces[nmax + b] = fy;
            a.forces[2 * nmax + b] = fz;
        }
        if (bad) atomicOr(s_bad, 1);
        bar_sync(bar, GT);
        if (gtid == 0) {
            if (*s_overflow) a.sys[slot].overflow = 1;
            a.sys[slot].eval_status = *s_bad ? kBatchStatusBlownUp : 0;
        }
    }
    if (ENERGY) {
#pragma unroll
        for (int k = 0; k < kNumSlots; ++k) {
            const double v = warp_sum_d(ea.e[k]);
            if (lane == 0 && v != 0.0) atomicAdd(&s_energy[k], v);
        }
        bar_sync(bar, GT);
        if (gtid < kNumSlots) a.energy[(size_t)slot * kNumSlots + gtid] = s_energy[gtid];
    }
}

template <int THREADS, int TERMS, bool LABELS, bool ENERGY, bool INTEGRATE>
__global__ void __launch_bounds__(THREADS, 1) k_batch(BatchArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    // per-group state (group 0 only until the split)
    __shared__ int s_claim[2];
    __shared__ int s_move[2][2];
    __shared__ int s_overflow[2];
    __shared__ int s_bad[2];
    __shared__ double s_energy[2][kNumSlots];
    __shared__ int s_item[2];
    const int tid = threadIdx.x;

    // Whole-CTA phase: every claimed system runs on all THREADS threads
    // (barrier 0).  When the CTA claims a system of at most split_beads
    // beads (capped on the host so that it fits half of the shared memory),
    // and the launch has at least two systems per CTA, it leaves this loop
    // with that system: claims come largest first, so every later system is
    // small too.  Every thread takes the same branch, right after a CTA-wide
    // barrier.
    int split_q = -1;
    while (true) {
        if (tid == 0) {
            s_claim[0] = atomicAdd(a.head, 1);
            s_move[0][0] = 0;
            s_move[0][1] = 0;
            s_overflow[0] = 0;
            s_bad[0] = 0;
        }
        if (ENERGY && tid < kNumSlots) s_energy[0][tid] = 0.0;
        __syncthreads();
        const int q = s_claim[0];
        if (q >= a.n_order) return;
        const int slot = a.order[q];
        const BatchSys& R = a.sys[slot];
        if (INTEGRATE && R.status != 0) {  // blew up earlier: not advanced again
            __syncthreads();  // every thread has read s_claim before it is rewritten
            continue;
        }
        if (R.n <= a.split_beads && a.n_order >= 2 * (int)gridDim.x) {
            split_q = q;
            break;
        }
        run_system<THREADS, TERMS, LABELS, ENERGY, INTEGRATE>(a, q, slot, tid, 0, smem, a.smem_bytes, s_move[0],
                                                              &s_overflow[0], &s_bad[0], s_energy[0], &s_item[0]);
        __syncthreads();
    }

    // Split phase, for the rest of the launch: two groups of THREADS / 2
    // threads, each with half of the shared memory and its own named barrier
    // (1 + g), each claiming and advancing its own systems; no barrier spans
    // both groups.  Group 0 starts with the system the CTA claimed (its words
    // were reset at that claim).  A system's results do not depend on the
    // threads that run it (the pair split depends on its bead count alone),
    // so they do not depend on the split either.
    constexpr int GT = THREADS / 2;
    const int g = tid / GT, gtid = tid - g * GT;
    const size_t half = (a.smem_bytes / 2) & ~(size_t)255;
    unsigned char* gsmem = smem + (size_t)g * half;
    bool first = g == 0;
    while (true) {
        if (!first) {
            if (gtid == 0) {
                s_claim[g] = atomicAdd(a.head, 1);
                s_move[g][0] = 0;
                s_move[g][1] = 0;
                s_overflow[g] = 0;
                s_bad[g] = 0;
            }
            if (ENERGY && gtid < kNumSlots) s_energy[g][gtid] = 0.0;
            bar_sync(1 + g, GT);
        }
        const int q = first ? split_q : s_claim[g];
        first = false;
        if (q >= a.n_order) return;
        const int slot = a.order[q];
        if (INTEGRATE && a.sys[slot].status != 0) {
            bar_sync(1 + g, GT);
            continue;
        }
        run_system<GT, TERMS, LABELS, ENERGY, INTEGRATE>(a, q, slot, gtid, 1 + g, gsmem, half, s_move[g],
                                                         &s_overflow[g], &s_bad[g], s_energy[g], &s_item[g]);
        bar_sync(1 + g, GT);
    }
}

__global__ void k_batch_velocity_init(int n, long long off, const float* __restrict__ invm,
                                      float kT, uint32_t seed, float* vx, float* vy, float* vz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float im = invm[i];
    const float3 g = gaussian3(seed, 1u, (uint32_t)i, 0ull, kPurposeVelocityInit);
    const float s = im > 0.f ? sqrtf(kT * im) : 0.f;
    vx[off + i] = s * g.x;
    vy[off + i] = s * g.y;
    vz[off + i] = s * g.z;
}

// Persistent launch: as many CTAs as fit, each given an equal share of the
// SM's shared memory (the state needs `smem`; the rest holds neighbour
// lists).
template <typename Fn>
// smem: shared memory the largest system needs; want: the share to aim
// for (state + bonded records + the list budget), 0 = all that fits.
void launch_persistent(Fn fn, int threads, BatchArgs a, int max_grid, size_t smem,
                       cudaStream_t s, int num_sms, size_t want) {
    // The kernel's shared-memory opt-in and its occupancy at this smem
    // size, looked up once per (kernel, device, size): the runtime queries
    // cost tens of microseconds per launch otherwise.
    struct Shape {
        int max_dyn, per_sm_smem, per_sm;
    };
    static std::mutex mu;
    static std::map<std::tuple<const void*, int, size_t, int>, Shape> cache;
    int dev = 0;
    OCM_CK(cudaGetDevice(&dev));
    Shape sh{};
    {
        std::lock_guard<std::mutex> lock(mu);
        const auto key = std::make_tuple(reinterpret_cast<const void*>(fn), dev, smem, threads);
        auto it = cache.find(key);
        if (it == cache.end()) {
            int optin = 0;
            OCM_CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
            OCM_CK(cudaDeviceGetAttribute(&sh.per_sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
            cudaFuncAttributes fa{};
            OCM_CK(cudaFuncGetAttributes(&fa, fn));
            sh.max_dyn = optin - (int)fa.sharedSizeBytes;
            OCM_CK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, sh.max_dyn));
            OCM_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&sh.per_sm, fn, threads, smem));
            it = cache.emplace(key, sh).first;
        }
        sh = it->second;
    }
    const int max_dyn = sh.max_dyn, per_sm_smem = sh.per_sm_smem;
    const int per_sm = sh.per_sm;
    if (per_sm < 1) throw Error(6, "[error] batched kernel does not fit on an SM");
    size_t share = (size_t)per_sm_smem / per_sm;
    share = share > 2048 ? share - 2048 : share;  // static + reserved per block
    share = std::min<size_t>(share, (size_t)max_dyn);
    if (want > 0) share = std::min(share, want);
    share = std::max(share, smem) & ~(size_t)15;
    a.smem_bytes = share;
    if (a.split_beads > 0) {
        // a group's system must fit half of the share (state of its beads,
        // the cluster arrays for the largest system, the pair-split offsets)
        const size_t half = (share / 2) & ~(size_t)255;
        const int fit = half > kFixedBytes ? (int)((half - kFixedBytes) / (size_t)a.split_bead_bytes) & ~31 : 0;
        a.split_beads = std::min(a.split_beads, fit);
    }
    const int grid = std::max(1, std::min(max_grid, num_sms * per_sm));
    fn<<<grid, threads, share, s>>>(a);
    OCM_CK(cudaGetLastError());
}

template <int THREADS, int TERMS, bool LABELS>
void launch_batch_t(const BatchArgs& a, int max_grid, size_t smem, cudaStream_t s, bool integrate,
                    bool energy, int num_sms, size_t lkib) {
    if (integrate)
        launch_persistent(k_batch<THREADS, TERMS, LABELS, false, true>, THREADS, a, max_grid, smem, s, num_sms, lkib);
    else if (energy)
        launch_persistent(k_batch<THREADS, TERMS, LABELS, true, false>, THREADS, a, max_grid, smem, s, num_sms, lkib);
    else
        launch_persistent(k_batch<THREADS, TERMS, LABELS, false, false>, THREADS, a, max_grid, smem, s, num_sms, lkib);
}

template <int TERMS, bool LABELS>
void launch_batch_threads(int threads, const BatchArgs& a, int grid, size_t smem, cudaStream_t s,
                          bool integrate, bool energy, int num_sms, size_t lkib) {
    switch (threads) {
        case 256: launch_batch_t<256, TERMS, LABELS>(a, grid, smem, s, integrate, energy, num_sms, lkib); break;
        case 512: launch_batch_t<512, TERMS, LABELS>(a, grid, smem, s, integrate, energy, num_sms, lkib); break;
        default: launch_batch_t<1024, TERMS, LABELS>(a, grid, smem, s, integrate, energy, num_sms, lkib); break;
    }
}

int64_t align_up(int64_t v, int64_t a) { return (v + a - 1) / a * a; }

// The bonded terms of one system in kernel order.  A term is chain-local
// when its beads are consecutive chain positions (bond b, b+1; angle b..b+2;
// dihedral b..b+3, either direction; angles and dihedrals are reversed to
// increasing order, which leaves the angle and the torsion unchanged).
// Chain-local terms come first, sorted by their first bead (stable, so
// terms on the same beads keep their order), with per-bead start indices;
// every other term is listed in the gather entries of each of its beads
// (type << 30 | role << 28 | term index).
struct BondedPlan {
    std::vector<BondTerm> bonds;
    std::vector<AngleTerm> angles;
    std::vector<DihedralTerm> dihedrals;
    std::vector<uint16_t> cb, ca, cd, gs;  // n + 1 each
    std::vector<uint32_t> gl;
};

BondedPlan plan_bonded(const CompiledSystem& c) {
    const int64_t n = c.n;
    BondedPlan P;
    std::vector<BondTerm> ob;
    std::vector<AngleTerm> oa;
    std::vector<DihedralTerm> od;
    std::vector<std::pair<int64_t, BondTerm>> chb;
    std::vector<std::pair<int64_t, AngleTerm>> cha;
    std::vector<std::pair<int64_t, DihedralTerm>> chd;
    for (BondTerm t : c.bonds) {
        if (t.i > t.j) std::swap(t.i, t.j);
        if (t.j == t.i + 1) chb.emplace_back(t.i, t);
        else ob.push_back(t);
    }
    for (AngleTerm t : c.angles) {
        if (t.i > t.k) std::swap(t.i, t.k);
        if (t.j == t.i + 1 && t.k == t.i + 2) cha.emplace_back(t.i, t);
        else oa.push_back(t);
    }
    for (DihedralTerm t : c.dihedrals) {
        if (t.i == t.j + 1 && t.j == t.k + 1 && t.k == t.l + 1) {
            std::swap(t.i, t.l);
            std::swap(t.j, t.k);
        }
        if (t.j == t.i + 1 && t.k == t.i + 2 && t.l == t.i + 3) chd.emplace_back(t.i, t);
        else od.push_back(t);
    }
    auto by_start = [](const auto& a, const auto& b) { return a.first < b.first; };
    std::stable_sort(chb.begin(), chb.end(), by_start);
    std::stable_sort(cha.begin(), cha.end(), by_start);
    std::stable_sort(chd.begin(), chd.end(), by_start);
    auto starts = [n](const auto& v) {
        std::vector<uint16_t> s(n + 1, 0);
        std::vector<int64_t> cnt(n + 1, 0);
        for (const auto& e : v) ++cnt[e.first + 1];
        for (int64_t b = 0; b < n; ++b) cnt[b + 1] += cnt[b];
        for (int64_t b = 0; b <= n; ++b) s[b] = (uint16_t)cnt[b];
        return s;
    };
    P.cb = starts(chb);
    P.ca = starts(cha);
    P.cd = starts(chd);
    for (auto& e : chb) P.bonds.push_back(e.second);
    for (auto& e : cha) P.angles.push_back(e.second);
    for (auto& e : chd) P.dihedrals.push_back(e.second);
    std::vector<std::vector<uint32_t>> g(n);
    auto entry = [](uint32_t type, uint32_t role, size_t idx) { return type << 30 | role << 28 | (uint32_t)idx; };
    for (const BondTerm& t : ob) {
        const size_t k = P.bonds.size();
        P.bonds.push_back(t);
        g[t.i].push_back(entry(0, 0, k));
        g[t.j].push_back(entry(0, 1, k));
    }
    for (const AngleTerm& t : oa) {
        const size_t k = P.angles.size();
        P.angles.push_back(t);
        g[t.i].push_back(entry(1, 0, k));
        g[t.j].push_back(entry(1, 1, k));
        g[t.k].push_back(entry(1, 2, k));
    }
    for (const DihedralTerm& t : od) {
        const size_t k = P.dihedrals.size();
        P.dihedrals.push_back(t);
        g[t.i].push_back(entry(2, 0, k));
        g[t.j].push_back(entry(2, 1, k));
        g[t.k].push_back(entry(2, 2, k));
        g[t.l].push_back(entry(2, 3, k));
    }
    P.gs.assign(n + 1, 0);
    for (int64_t b = 0; b < n; ++b) {
        P.gl.insert(P.gl.end(), g[b].begin(), g[b].end());
        if (P.gl.size() > 0xFFFF) throw Error(6, "[error] too many bonded terms per system for the batched path");
        P.gs[b + 1] = (uint16_t)P.gl.size();
    }
    if (P.bonds.size() > 0xFFFF || P.angles.size() > 0xFFFF || P.dihedrals.size() > 0xFFFF)
        throw Error(6, "[error] too many bonded terms per system for the batched path");
    return P;
}

struct BlobLayout {
    int64_t size = 0;
    int off_p0, off_p1, off_lab, off_invm, off_ex_start, off_ex;
    int off_bonded, bonded_bytes, rb_p, rb_ij, ra_ij, ra_k, rd, rgd, rfla, rfld;
    int rcb, rca, rcd, rgs, rgl;
};

BlobLayout blob_layout(const CompiledSystem& c, const BondedPlan& P) {
    BlobLayout L{};
    const int64_t n = c.n;
    int64_t o = 0;
    auto take = [&](int64_t bytes) {
        const int64_t at = o;
        o = align_up(o + bytes, 16);
        return (int)at;
    };
    L.off_p0 = take(16 * n);
    L.off_p1 = take(16 * n);
    L.off_lab = take(4 * n);
    L.off_invm = take(4 * n);
    // bonded region: bond params (float4) | bond indices (u32) | angle
    // indices (uint2) | angle k (f32) | dihedral records (uint4) | Gaussian
    // dihedral parameters | FLA | FLD | chain starts (3 x u16) | gather
    // starts (u16) | gather entries (u32)
    L.off_bonded = (int)o;
    const int64_t nb = (int64_t)P.bonds.size(), na = (int64_t)P.angles.size(),
                  nd = (int64_t)P.dihedrals.size();
    L.rb_p = take(16 * nb) - L.off_bonded;
    L.rb_ij = take(4 * nb) - L.off_bonded;
    L.ra_ij = take(8 * na) - L.off_bonded;
    L.ra_k = take(4 * na) - L.off_bonded;
    L.rd = take(16 * nd) - L.off_bonded;
    int64_t ngd = 0;
    for (const auto& t : P.dihedrals) ngd += t.kind == kDihGauss ? 1 : 0;
    L.rgd = take(8 * ngd) - L.off_bonded;
    L.rfla = take((int64_t)sizeof(FlaTable) * c.fla.size()) - L.off_bonded;
    L.rfld = take((int64_t)sizeof(FldTable) * c.fld.size()) - L.off_bonded;
    L.rcb = take(2 * (n + 1)) - L.off_bonded;
    L.rca = take(2 * (n + 1)) - L.off_bonded;
    L.rcd = take(2 * (n + 1)) - L.off_bonded;
    L.rgs = take(2 * (n + 1)) - L.off_bonded;
    L.rgl = take(4 * (int64_t)P.gl.size()) - L.off_bonded;
    L.bonded_bytes = (int)(o - L.off_bonded);
    L.off_ex_start = take(4 * (n + 1));
    L.off_ex = take(4 * (int64_t)c.ex_j.size());
    L.size = align_up(o, 256);
    return L;
}

constexpr float kBatchSkin = 0.3f;  // nm

// Entries per bead of a system's neighbour list: the largest count within
// the list cutoff at admission, with head-room for compaction.
int initial_list_capacity(const CompiledSystem& c, const double* pos) {
    const int64_t n = c.n;
    if (c.pc.terms == 0) return 1;
    const double cut = std::sqrt((double)c.pc.list_rc2) + kBatchSkin;
    const double cut2 = cut * cut;
    int mx = 0;
    for (int64_t i = 0; i < n; ++i) {
        int cnt = 0;
        for (int64_t j = 0; j < n; ++j) {
            if (j == i) continue;
            const double dx = pos[3 * j] - pos[3 * i], dy = pos[3 * j + 1] - pos[3 * i + 1],
                         dz = pos[3 * j + 2] - pos[3 * i + 2];
            cnt += dx * dx + dy * dy + dz * dz < cut2;
        }
        mx = std::max(mx, cnt);
    }
    const int cap = (int)std::ceil(1.25 * mx) + 16;
    return (int)std::min<int64_t>(std::max<int64_t>(1, n - 1), align_up(cap, 4));
}

void check_batchable(const CompiledSystem& c, int nmax) {
    if (c.n <= 0) throw Error(1, "[error] system has no particles");
    if (c.n > nmax)
        throw Error(3, "[error] system of " + std::to_string(c.n) +
                           " beads exceeds the batch's per-system limit " + std::to_string(nmax));
    if (c.periodic) throw Error(6, "[error] the batched path runs non-periodic systems");
    for (const auto& b : c.bonds)
        if (b.periodic) throw Error(6, "[error] the batched path runs non-periodic systems");
}

}  // namespace

// ---------------------------------------------------------------------------
int64_t RangeAllocator::alloc(int64_t size, int64_t align) {
    if (size <= 0) size = 1;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
        const int64_t off = it->first, sz = it->second;
        const int64_t a = align_up(off, align);
        if (a + size <= off + sz) {
            free_.erase(it);
            if (a > off) free_[off] = a - off;
            if (a + size < off + sz) free_[a + size] = off + sz - (a + size);
            return a;
        }
    }
    return -1;
}

void RangeAllocator::release(int64_t off, int64_t size) {
    if (size <= 0) size = 1;
    auto it = free_.emplace(off, size).first;
    auto next = std::next(it);
    if (next != free_.end() && it->first + it->second == next->first) {
        it->second += next->second;
        free_.erase(next);
    }
    if (it != free_.begin()) {
        auto prev = std::prev(it);
        if (prev->first + prev->second == it->first) {
            prev->second += it->second;
            free_.erase(it);
        }
    }
}

// ---------------------------------------------------------------------------
BatchEngine::BatchEngine(int device, int64_t max_systems, int64_t max_beads, int32_t nmax)
    : device_(device), max_systems_(max_systems), max_beads_(max_beads) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
        throw Error(2, "[error] no CUDA device is available");
    if (device < 0 || device >= count) throw Error(1, "[error] invalid device index");
    if (max_systems <= 0 || max_beads <= 0 || nmax <= 0) throw Error(1, "[error] invalid batch capacity");
    if (nmax > 32 * kMaxClusters)
        throw Error(6, "[error] at most " + std::to_string(32 * kMaxClusters) + " beads per system");
    OCM_CK(cudaSetDevice(device));
    nmax_ = (int)align_up(nmax, 32);
    OCM_CK(cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, device));
    int optin = 0;
    OCM_CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
    if ((int64_t)smem_bytes(nmax_, false) > optin)
        throw Error(6, "[error] per-system bead limit does not fit in shared memory");
    OCM_CK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    OCM_CK(cudaStreamCreateWithFlags(&copy_stream_, cudaStreamNonBlocking));
    OCM_CK(cudaEventCreate(&ev0_));
    OCM_CK(cudaEventCreate(&ev1_));
    OCM_CK(cudaEventCreateWithFlags(&ev_copy_, cudaEventDisableTiming));
    slots_.resize(max_systems);
    sys_host_.resize(max_systems);
    std::memset(sys_host_.data(), 0, sizeof(BatchSys) * max_systems);
    beads_.reset(max_beads);
    // Static blobs: per bead ~ 40 B of parameters + ~4 terms of 24 B, plus
    // the cluster-pair mask tables.
    const int64_t blob_cap = max_beads * 256 + max_systems * 8192;
    blob_.reset(blob_cap);
    x_.alloc(max_beads); y_.alloc(max_beads); z_.alloc(max_beads);
    vx_.alloc(max_beads); vy_.alloc(max_beads); vz_.alloc(max_beads);
    blob_dev_.alloc(blob_cap);
    const int64_t list_cap = max_beads * 256 + max_systems * 1024;
    list_alloc_.reset(list_cap);
    lists_.alloc(list_cap);
    OCM_CK(cudaMallocHost(&h_overflow_, sizeof(int) * max_systems));
    std::memset(h_overflow_, 0, sizeof(int) * max_systems);
    OCM_CK(cudaMallocHost(&h_status_, sizeof(int) * max_systems));
    std::memset(h_status_, 0, sizeof(int) * max_systems);
    OCM_CK(cudaMallocHost(&h_check_, sizeof(int)));
    check_.alloc(1);
    sys_.alloc(max_systems);
    OCM_CK(cudaMemset(sys_.p, 0, sizeof(BatchSys) * max_systems));
    order_.alloc(max_systems);
    order_k_.alloc(max_systems);
    head_.alloc(1);
    energy_.alloc(max_systems * kNumSlots);
    forces_.alloc(3 * nmax_);
}

BatchEngine::~BatchEngine() {
    cudaSetDevice(device_);
    if (stream_) cudaStreamSynchronize(stream_);
    if (copy_stream_) cudaStreamSynchronize(copy_stream_);
    if (ev0_) cudaEventDestroy(ev0_);
    if (ev1_) cudaEventDestroy(ev1_);
    if (ev_copy_) cudaEventDestroy(ev_copy_);
    if (h_overflow_) cudaFreeHost(h_overflow_);
    if (h_status_) cudaFreeHost(h_status_);
    if (h_check_) cudaFreeHost(h_check_);
    if (stream_) cudaStreamDestroy(stream_);
    if (copy_stream_) cudaStreamDestroy(copy_stream_);
}

// Shared memory of the per-system state: kBeadBytes per bead
// (kBeadBytesGeneral with the general pair terms) and kFixedBytes.
size_t BatchEngine::smem_bytes(int nmax, bool general) const {
    return (size_t)nmax * (general ? kBeadBytesGeneral : kBeadBytes) + kFixedBytes;
}

int64_t BatchEngine::footprint(const SystemDesc& d) {
    CompiledSystem c = compile_system(d);
    const BondedPlan P = plan_bonded(c);
    const BlobLayout L = blob_layout(c, P);
    return L.size + c.n * (3 * 8 + 3 * 4) + (int64_t)sizeof(BatchSys);
}

void BatchEngine::set_list_smem(int kib) {
    if (kib < -1 || kib > 228) throw Error(1, "[error] list shared memory must be -1 or 0..228 KiB");
    list_smem_kib_ = kib;
}

void BatchEngine::set_split(int beads) {
    if (beads < 0 || beads > 32 * kMaxClusters) throw Error(1, "[error] split bead limit must be in 0..2048");
    split_beads_ = beads;
}

void BatchEngine::set_threads(int threads) {
    if (threads != 256 && threads != 512 && threads != 1024)
        throw Error(1, "[error] threads per CTA must be 256, 512 or 1024");
    threads_ = threads;
}

int64_t BatchEngine::admit(const SystemDesc& d, const double* pos, const double* vel, double T,
                           double friction, double dt, int32_t seed, int64_t n_steps, int64_t steps_done) {
    OCM_CK(cudaSetDevice(device_));
    if (n_steps < 0) throw Error(1, "[error] negative step count");
    if (steps_done < 0 || steps_done > n_steps)
        throw Error(1, "[error] steps already done must lie in [0, step count]");
    if (!(dt > 0) || !(friction >= 0) || !(T >= 0)) throw Error(1, "[error] invalid integrator parameters");
    CompiledSystem c = compile_system(d);
    check_batchable(c, nmax_);
    const int64_t n = c.n;
    for (int64_t i = 0; i < 3 * n; ++i)
        if (!std::isfinite(pos[i])) throw Error(7, "[error] non-finite position");
    int64_t slot = -1;
    for (int64_t s = 0; s < max_systems_; ++s)
        if (!slots_[s].used) {
            slot = s;
            break;
        }
    if (slot < 0) throw Error(3, "[error] no free slot in the batch");
    const BondedPlan P = plan_bonded(c);
    const BlobLayout L = blob_layout(c, P);
    const int npad = (int)align_up(n, 32);
    const int maxn = initial_list_capacity(c, pos);
    const int64_t boff = beads_.alloc(n, 1);
    if (boff < 0) throw Error(3, "[error] batch bead capacity exhausted");
    const int64_t blob_off = blob_.alloc(L.size, 256);
    if (blob_off < 0) {
        beads_.release(boff, n);
        throw Error(3, "[error] batch parameter memory exhausted");
    }
    const int64_t list_size = (int64_t)maxn * npad;
    const int64_t list_off = list_alloc_.alloc(list_size, 64);
    if (list_off < 0) {
        beads_.release(boff, n);
        blob_.release(blob_off, L.size);
        throw Error(3, "[error] batch neighbour-list memory exhausted");
    }
    // host blob
    std::vector<unsigned char> blob(L.size, 0);
    auto put = [&](int off, const void* src, size_t bytes) {
        if (bytes) std::memcpy(blob.data() + off, src, bytes);
    };
    put(L.off_p0, c.p0.data(), 16 * n);
    put(L.off_p1, c.p1.data(), 16 * n);
    put(L.off_lab, c.labels.data(), 4 * n);
    put(L.off_invm, c.inv_mass.data(), 4 * n);
    {
        // compact bonded records (bead indices < 2048 fit 16 bits)
        std::vector<float4> bp(P.bonds.size());
        std::vector<uint32_t> bij(P.bonds.size());
        for (size_t b = 0; b < P.bonds.size(); ++b) {
            const BondTerm& t = P.bonds[b];
            bp[b] = make_float4(t.p0, t.p1, t.r0sq_hi, t.r0sq_lo);
            bij[b] = (uint32_t)t.i | ((uint32_t)t.j << 16) | ((uint32_t)t.kind << 30);
        }
        std::vector<uint2> aij(P.angles.size());
        std::vector<float> ak(P.angles.size());
        for (size_t b = 0; b < P.angles.size(); ++b) {
            const AngleTerm& t = P.angles[b];
            aij[b] = make_uint2((uint32_t)t.i | ((uint32_t)t.j << 16), (uint32_t)t.k | ((uint32_t)t.table << 16));
            ak[b] = t.kk;
        }
        // dihedral record: FLD table index, or (bit 31 of .x set) the index
        // of the Gaussian dihedral's (theta0, 1 / (2 sigma^2))
        std::vector<uint4> dr(P.dihedrals.size());
        std::vector<float2> gd;
        for (size_t b = 0; b < P.dihedrals.size(); ++b) {
            const DihedralTerm& t = P.dihedrals[b];
            uint32_t kb;
            std::memcpy(&kb, &t.kk, 4);
            const bool gauss = t.kind == kDihGauss;
            uint32_t third = (uint32_t)t.table;
            if (gauss) {
                third = (uint32_t)gd.size();
                gd.push_back(make_float2(t.theta0, t.inv2s2));
            }
            dr[b] = make_uint4((uint32_t)t.i | ((uint32_t)t.j << 16) | (gauss ? 0x80000000u : 0u),
                               (uint32_t)t.k | ((uint32_t)t.l << 16), third, kb);
        }
        const int ob = L.off_bonded;
        put(ob + L.rb_p, bp.data(), 16 * bp.size());
        put(ob + L.rb_ij, bij.data(), 4 * bij.size());
        put(ob + L.ra_ij, aij.data(), 8 * aij.size());
        put(ob + L.ra_k, ak.data(), 4 * ak.size());
        put(ob + L.rd, dr.data(), 16 * dr.size());
        put(ob + L.rgd, gd.data(), 8 * gd.size());
        put(ob + L.rfla, c.fla.data(), sizeof(FlaTable) * c.fla.size());
        put(ob + L.rfld, c.fld.data(), sizeof(FldTable) * c.fld.size());
        put(ob + L.rcb, P.cb.data(), 2 * P.cb.size());
        put(ob + L.rca, P.ca.data(), 2 * P.ca.size());
        put(ob + L.rcd, P.cd.data(), 2 * P.cd.size());
        put(ob + L.rgs, P.gs.data(), 2 * P.gs.size());
        put(ob + L.rgl, P.gl.data(), 4 * P.gl.size());
    }
    {
        std::vector<int32_t> ex(c.ex_j.size());
        for (size_t e = 0; e < ex.size(); ++e) ex[e] = c.ex_j[e] | ((int32_t)c.ex_bits[e] << 24);
        put(L.off_ex_start, c.ex_start.data(), 4 * c.ex_start.size());
        put(L.off_ex, ex.data(), 4 * ex.size());
    }

    BatchSys R{};
    R.bead_off = boff;
    R.blob_off = blob_off;
    R.n = (int)n;
    R.nt = (int)((n + 31) / 32);
    R.n_bonds = (int)P.bonds.size();
    R.n_angles = (int)P.angles.size();
    R.n_dih = (int)P.dihedrals.size();
    R.off_p0 = L.off_p0; R.off_p1 = L.off_p1; R.off_lab = L.off_lab; R.off_invm = L.off_invm;
    R.off_bonded = L.off_bonded; R.bonded_bytes = L.bonded_bytes;
    R.rb_p = L.rb_p; R.rb_ij = L.rb_ij; R.ra_ij = L.ra_ij; R.ra_k = L.ra_k; R.rd = L.rd; R.rgd = L.rgd;
    R.rfla = L.rfla; R.rfld = L.rfld;
    R.rcb = L.rcb; R.rca = L.rca; R.rcd = L.rcd; R.rgs = L.rgs; R.rgl = L.rgl;
    R.off_ex_start = L.off_ex_start; R.off_ex = L.off_ex;
    R.skin = kBatchSkin;
    R.maxn = maxn;
    R.list_off = list_off;
    R.active = 1;
    R.pc = c.pc;
    const double vscale = std::exp(-friction * dt);
    const double fscale = friction == 0 ? dt : (1.0 - vscale) / friction;
    const double kT = constant::boltz * T;
    R.lc.vscale = (float)vscale;
    R.lc.fscale = (float)fscale;
    R.lc.noise = (float)std::sqrt(kT * (1.0 - vscale * vscale));
    R.lc.dt = (float)dt;
    R.lc.seed = (uint32_t)seed;
    R.lc.stream = 0u;
    R.steps_done = (unsigned long long)steps_done;
    R.steps_target = (unsigned long long)n_steps;

    std::vector<double> px(n), py(n), pz(n);
    for (int64_t i = 0; i < n; ++i) {
        px[i] = pos[3 * i];
        py[i] = pos[3 * i + 1];
        pz[i] = pos[3 * i + 2];
    }
    cudaStream_t s = copy_stream_;
    OCM_CK(cudaMemcpyAsync(blob_dev_.p + blob_off, blob.data(), L.size, cudaMemcpyHostToDevice, s));
    OCM_CK(cudaMemcpyAsync(x_.p + boff, px.data(), n * sizeof(double), cudaMemcpyHostToDevice, s));
    OCM_CK(cudaMemcpyAsync(y_.p + boff, py.data(), n * sizeof(double), cudaMemcpyHostToDevice, s));
    OCM_CK(cudaMemcpyAsync(z_.p + boff, pz.data(), n * sizeof(double), cudaMemcpyHostToDevice, s));
    if (vel) {
        std::vector<float> vx(n), vy(n), vz(n);
        for (int64_t i = 0; i < n; ++i) {
            vx[i] = (float)vel[3 * i];
            vy[i] = (float)vel[3 * i + 1];
            vz[i] = (float)vel[3 * i + 2];
        }
        OCM_CK(cudaMemcpyAsync(vx_.p + boff, vx.data(), n * sizeof(float), cudaMemcpyHostToDevice, s));
        OCM_CK(cudaMemcpyAsync(vy_.p + boff, vy.data(), n * sizeof(float), cudaMemcpyHostToDevice, s));
        OCM_CK(cudaMemcpyAsync(vz_.p + boff, vz.data(), n * sizeof(float), cudaMemcpyHostToDevice, s));
    } else {
        k_batch_velocity_init<<<(int)((n + 255) / 256), 256, 0, s>>>(
            (int)n, boff, reinterpret_cast<const float*>(blob_dev_.p + blob_off + L.off_invm),
            (float)kT, (uint32_t)seed, vx_.p, vy_.p, vz_.p);
        OCM_CK(cudaGetLastError());
    }
    OCM_CK(cudaMemcpyAsync(sys_.p + slot, &R, sizeof(BatchSys), cudaMemcpyHostToDevice, s));
    // pageable copies above are complete on return except the record, keep
    // the host objects alive until then
    OCM_CK(cudaStreamSynchronize(s));
    OCM_CK(cudaEventRecord(ev_copy_, s));

    Slot& S = slots_[slot];
    S.used = true;
    S.bead_off = boff;
    S.n = n;
    S.blob_off = blob_off;
    S.blob_size = L.size;
    S.steps_target = (uint64_t)n_steps;
    S.steps_done = (uint64_t)steps_done;
    S.list_off = list_off;
    S.list_size = list_size;
    S.maxn = maxn;
    S.terms = c.pc.terms;
    S.labels = c.pc.uses_labels != 0;
    for (int k = 0; k < kNumSlots; ++k) S.slot_group[k] = c.slot_group[k];
    const double nt = (double)R.nt;
    S.cost = nt * (nt + 1) / 2 + 0.05 * (double)n;
    sys_host_[slot] = R;
    return slot;
}

void BatchEngine::launch(bool integrate, bool energy, int k, const std::vector<int32_t>& order,
                         cudaStream_t s, const std::vector<int32_t>* order_k) {
    bool general = false;
    int terms = 0;
    size_t bonded_max = 0;
    for (int32_t q : order) {
        terms |= slots_[q].terms;
        general = general || slots_[q].labels;
        bonded_max = std::max(bonded_max, (size_t)sys_host_[q].bonded_bytes);
    }
    if (terms & ~(kTermEXV | kTermDH)) general = true;
    const size_t smem = smem_bytes(nmax_, general);
    const size_t want = list_smem_kib_ >= 0 ? smem + bonded_max + (size_t)list_smem_kib_ * 1024 : 0;
    int optin = 0;
    OCM_CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device_));
    if ((int64_t)smem > optin)
        throw Error(6, "[error] these systems need more shared memory than one SM offers; "
                       "create the batch with a smaller per-system bead limit");
    OCM_CK(cudaMemcpyAsync(order_.p, order.data(), order.size() * sizeof(int32_t),
                           cudaMemcpyHostToDevice, s));
    if (order_k)
        OCM_CK(cudaMemcpyAsync(order_k_.p, order_k->data(), order_k->size() * sizeof(int32_t),
                               cudaMemcpyHostToDevice, s));
    OCM_CK(cudaMemsetAsync(head_.p, 0, sizeof(int32_t), s));
    BatchArgs a{};
    a.sys = sys_.p;
    a.order = order_.p;
    a.order_k = order_k ? order_k_.p : nullptr;
    a.n_order = (int)order.size();
    a.head = head_.p;
    a.x = x_.p; a.y = y_.p; a.z = z_.p;
    a.vx = vx_.p; a.vy = vy_.p; a.vz = vz_.p;
    a.blob = blob_dev_.p;
    a.k = k;
    a.nmax = nmax_;
    a.energy = energy_.p;
    a.forces = forces_.p;
    a.lists = lists_.p;
    a.slots_enabled = 0xffffffffu;
    a.split_beads = integrate ? split_beads_ : 0;
    a.split_bead_bytes = general ? kBeadBytesGeneral : kBeadBytes;
    const int grid = (int)order.size();
    if (general)
        launch_batch_threads<15, true>(threads_, a, grid, smem, s, integrate, energy, num_sms_, want);
    else
        launch_batch_threads<kTermEXV | kTermDH, false>(threads_, a, grid, smem, s, integrate, energy, num_sms_,
                                                         want);
}

void BatchEngine::run(int32_t k, bool sync) {
    OCM_CK(cudaSetDevice(device_));
    if (k <= 0) throw Error(1, "[error] steps per launch must be positive");
    // settle the previous launch first: list growth and systems that blew up
    grow_lists();
    std::vector<int32_t> order;
    for (int64_t s = 0; s < max_systems_; ++s)
        if (slots_[s].used && !slots_[s].failed && slots_[s].steps_done < slots_[s].steps_target)
            order.push_back((int32_t)s);
    std::stable_sort(order.begin(), order.end(),
                     [&](int32_t a, int32_t b) { return slots_[a].cost > slots_[b].cost; });
    // Balanced launches: the costliest system does k steps, every other one
    // as many more as its lower cost allows in the same time (a system's
    // trajectory does not depend on how its steps are split into launches).
    std::vector<int32_t> ks(order.size(), k);
    if (balanced_ && !order.empty()) {
        const double ref = step_cost(slots_[order.front()].n);
        for (size_t q = 0; q < order.size(); ++q)
            ks[q] = (int32_t)std::min<double>(64.0 * k, std::max(1.0, std::floor(k * ref / step_cost(slots_[order[q]].n))));
    }
    OCM_CK(cudaStreamWaitEvent(stream_, ev_copy_, 0));
    OCM_CK(cudaEventRecord(ev0_, stream_));
    if (!order.empty()) launch(true, false, k, order, stream_, balanced_ ? &ks : nullptr);
    OCM_CK(cudaEventRecord(ev1_, stream_));
    OCM_CK(cudaMemcpy2DAsync(h_overflow_, sizeof(int), &sys_.p[0].overflow, sizeof(BatchSys),
                             sizeof(int), max_systems_, cudaMemcpyDeviceToHost, stream_));
    OCM_CK(cudaMemcpy2DAsync(h_status_, sizeof(int), &sys_.p[0].status, sizeof(BatchSys),
                             sizeof(int), max_systems_, cudaMemcpyDeviceToHost, stream_));
    ran_ = true;
    for (size_t q = 0; q < order.size(); ++q) {
        Slot& S = slots_[order[q]];
        S.steps_done = std::min<uint64_t>(S.steps_target, S.steps_done + (uint64_t)ks[q]);
    }
    if (sync) OCM_CK(cudaStreamSynchronize(stream_));
}

double BatchEngine::last_run_ms() {
    OCM_CK(cudaSetDevice(device_));
    if (!ran_) return 0.0;
    OCM_CK(cudaEventSynchronize(ev1_));
    float ms = 0.f;
    OCM_CK(cudaEventElapsedTime(&ms, ev0_, ev1_));
    return ms;
}

// Waits for the last launch and takes note of systems that blew up in it:
// they stopped at the failing step, so their step counters come from the
// device, and they are not launched again.
void BatchEngine::sync_steps() {
    OCM_CK(cudaStreamSynchronize(stream_));
    if (!ran_) return;
    for (int64_t s = 0; s < max_systems_; ++s) {
        if (!slots_[s].used || slots_[s].failed || h_status_[s] == 0) continue;
        slots_[s].failed = true;
        unsigned long long done = 0;
        OCM_CK(cudaMemcpy(&done, &sys_.p[s].steps_done, sizeof(done), cudaMemcpyDeviceToHost));
        slots_[s].steps_done = done;
    }
}

void BatchEngine::load_state_device(int64_t slot, const double* x, const double* y, const double* z,
                                    const float* vx, const float* vy, const float* vz, uint64_t steps_done,
                                    uint64_t steps_target) {
    OCM_CK(cudaSetDevice(device_));
    if (slot < 0 || slot >= max_systems_ || !slots_[slot].used) throw Error(1, "[error] invalid slot");
    if (steps_done > steps_target) throw Error(1, "[error] steps already done exceed the step target");
    sync_steps();
    Slot& S = slots_[slot];
    const int64_t n = S.n, o = S.bead_off;
    cudaStream_t s = stream_;
    OCM_CK(cudaMemcpyAsync(x_.p + o, x, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    OCM_CK(cudaMemcpyAsync(y_.p + o, y, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    OCM_CK(cudaMemcpyAsync(z_.p + o, z, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    OCM_CK(cudaMemcpyAsync(vx_.p + o, vx, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
    OCM_CK(cudaMemcpyAsync(vy_.p + o, vy, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
    OCM_CK(cudaMemcpyAsync(vz_.p + o, vz, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
    BatchSys& R = sys_host_[slot];
    R.steps_done = steps_done;
    R.steps_target = steps_target;
    R.status = 0;
    BatchSys* dst = sys_.p + slot;
    OCM_CK(cudaMemcpyAsync(&dst->steps_done, &R.steps_done, 2 * sizeof(unsigned long long),
                           cudaMemcpyHostToDevice, s));
    OCM_CK(cudaMemcpyAsync(&dst->status, &R.status, sizeof(int), cudaMemcpyHostToDevice, s));
    OCM_CK(cudaStreamSynchronize(s));
    S.steps_done = steps_done;
    S.steps_target = steps_target;
    S.failed = false;
    h_status_[slot] = 0;
}

void BatchEngine::store_state_device(int64_t slot, double* x, double* y, double* z, float* vx, float* vy,
                                     float* vz) {
    OCM_CK(cudaSetDevice(device_));
    if (slot < 0 || slot >= max_systems_ || !slots_[slot].used) throw Error(1, "[error] invalid slot");
    sync_steps();
    const Slot& S = slots_[slot];
    const int64_t n = S.n, o = S.bead_off;
    cudaStream_t s = stream_;
    OCM_CK(cudaMemcpyAsync(x, x_.p + o, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    OCM_CK(cudaMemcpyAsync(y, y_.p + o, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    OCM_CK(cudaMemcpyAsync(z, z_.p + o, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    OCM_CK(cudaMemcpyAsync(vx, vx_.p + o, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
    OCM_CK(cudaMemcpyAsync(vy, vy_.p + o, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
    OCM_CK(cudaMemcpyAsync(vz, vz_.p + o, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
    OCM_CK(cudaStreamSynchronize(s));
}

int32_t BatchEngine::slot_status(int64_t slot) {
    OCM_CK(cudaSetDevice(device_));
    if (slot < 0 || slot >= max_systems_ || !slots_[slot].used) throw Error(1, "[error] invalid slot");
    sync_steps();
    return slots_[slot].failed ? 7 : 0;
}

// A list that overflowed made its system fall back to the tile sweep for
// the rest of that chunk (same results, more work); give it more room now.
void BatchEngine::grow_lists() {
    if (!ran_) return;
    sync_steps();
    for (int64_t s = 0; s < max_systems_; ++s) {
        if (!h_overflow_[s] || !slots_[s].used) continue;
        h_overflow_[s] = 0;
        Slot& S = slots_[s];
        const int npad = (int)align_up(S.n, 32);
        const int maxn = (int)std::min<int64_t>(std::max<int64_t>(1, S.n - 1), align_up(S.maxn * 3 / 2 + 8, 4));
        const int64_t size = (int64_t)maxn * npad;
        list_alloc_.release(S.list_off, S.list_size);
        const int64_t off = list_alloc_.alloc(size, 64);
        if (off < 0) {
            const int64_t back = list_alloc_.alloc(S.list_size, 64);
            (void)back;
            throw Error(3, "[error] batch neighbour-list memory exhausted while growing a list");
        }
        S.list_off = off;
        S.list_size = size;
        S.maxn = maxn;
        sys_host_[s].list_off = off;
        sys_host_[s].maxn = maxn;
        sys_host_[s].overflow = 0;
        BatchSys* dst = sys_.p + s;
        OCM_CK(cudaMemcpyAsync(&dst->list_off, &sys_host_[s].list_off, sizeof(long long),
                               cudaMemcpyHostToDevice, stream_));
        OCM_CK(cudaMemcpyAsync(&dst->maxn, &sys_host_[s].maxn, sizeof(int), cudaMemcpyHostToDevice, stream_));
        OCM_CK(cudaMemcpyAsync(&dst->overflow, &sys_host_[s].overflow, sizeof(int),
                               cudaMemcpyHostToDevice, stream_));
        OCM_CK(cudaStreamSynchronize(stream_));
    }
}

void BatchEngine::finished(int64_t* out, int64_t cap, int64_t* n_out) {
    OCM_CK(cudaSetDevice(device_));
    sync_steps();
    int64_t c = 0;
    for (int64_t s = 0; s < max_systems_; ++s) {
        if (!slots_[s].used || (!slots_[s].failed && slots_[s].steps_done < slots_[s].steps_target)) continue;
        if (out && c < cap) out[c] = s;
        ++c;
    }
    *n_out = c;
}

void BatchEngine::get_positions(int64_t slot, double* xyz) {
    OCM_CK(cudaSetDevice(device_));
    if (slot < 0 || slot >= max_systems_ || !slots_[slot].used) throw Error(1, "[error] invalid slot");
    sync_steps();
    const Slot& S = slots_[slot];
    std::vector<double> a(S.n), b(S.n), c(S.n);
    OCM_CK(cudaMemcpy(a.data(), x_.p + S.bead_off, S.n * sizeof(double), cudaMemcpyDeviceToHost));
    OCM_CK(cudaMemcpy(b.data(), y_.p + S.bead_off, S.n * sizeof(double), cudaMemcpyDeviceToHost));
    OCM_CK(cudaMemcpy(c.data(), z_.p + S.bead_off, S.n * sizeof(double), cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < S.n; ++i) {
        xyz[3 * i] = a[i];
        xyz[3 * i + 1] = b[i];
        xyz[3 * i + 2] = c[i];
    }
}

void BatchEngine::get_velocities(int64_t slot, double* v) {
    OCM_CK(cudaSetDevice(device_));
    if (slot < 0 || slot >= max_systems_ || !slots_[slot].used) throw Error(1, "[error] invalid slot");
    sync_steps();
    const Slot& S = slots_[slot];
    std::vector<float> a(S.n), b(S.n), c(S.n);
    OCM_CK(cudaMemcpy(a.data(), vx_.p + S.bead_off, S.n * sizeof(float), cudaMemcpyDeviceToHost));
    OCM_CK(cudaMemcpy(b.data(), vy_.p + S.bead_off, S.n * sizeof(float), cudaMemcpyDeviceToHost));
    OCM_CK(cudaMemcpy(c.data(), vz_.p + S.bead_off, S.n * sizeof(float), cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < S.n; ++i) {
        v[3 * i] = a[i];
        v[3 * i + 1] = b[i];
        v[3 * i + 2] = c[i];
    }
}

int64_t BatchEngine::steps_done(int64_t slot) {
    if (slot < 0 || slot >= max_systems_ || !slots_[slot].used) throw Error(1, "[error] invalid slot");
    sync_steps();
    return (int64_t)slots_[slot].steps_done;
}

void BatchEngine::get_state(int64_t slot, uint32_t groups, double* forces, double* energies) {
    OCM_CK(cudaSetDevice(device_));
    if (slot < 0 || slot >= max_systems_ || !slots_[slot].used) throw Error(1, "[error] invalid slot");
    const Slot& S = slots_[slot];
    uint32_t en = 0;
    for (int k = 0; k < kNumSlots; ++k)
        if (S.slot_group[k] >= 0 && ((groups >> S.slot_group[k]) & 1u)) en |= 1u << k;
    std::vector<int32_t> order{(int32_t)slot};
    OCM_CK(cudaStreamWaitEvent(stream_, ev_copy_, 0));
    OCM_CK(cudaMemsetAsync(energy_.p + slot * kNumSlots, 0, kNumSlots * sizeof(double), stream_));
    // The eval kernel reads slots_enabled from the args.
    {
        bool general = S.labels || (S.terms & ~(kTermEXV | kTermDH));
        const size_t smem = smem_bytes(nmax_, general);
        OCM_CK(cudaMemcpyAsync(order_.p, order.data(), sizeof(int32_t), cudaMemcpyHostToDevice, stream_));
        OCM_CK(cudaMemsetAsync(head_.p, 0, sizeof(int32_t), stream_));
        BatchArgs a{};
        a.sys = sys_.p; a.order = order_.p; a.n_order = 1; a.head = head_.p;
        a.x = x_.p; a.y = y_.p; a.z = z_.p; a.vx = vx_.p; a.vy = vy_.p; a.vz = vz_.p;
        a.blob = blob_dev_.p; a.k = 0; a.nmax = nmax_; a.energy = energy_.p; a.forces = forces_.p;
        a.lists = lists_.p;
        a.slots_enabled = en;
        const size_t want = list_smem_kib_ >= 0
                                ? smem + (size_t)sys_host_[slot].bonded_bytes + (size_t)list_smem_kib_ * 1024
                                : 0;
        if (general) launch_batch_threads<15, true>(threads_, a, 1, smem, stream_, false, true, num_sms_, want);
        else launch_batch_threads<kTermEXV | kTermDH, false>(threads_, a, 1, smem, stream_, false, true, num_sms_,
                                                              want);
    }
    std::vector<float> f(3 * nmax_);
    double e[kNumSlots];
    int bad = 0;
    OCM_CK(cudaMemcpyAsync(f.data(), forces_.p, 3 * nmax_ * sizeof(float), cudaMemcpyDeviceToHost, stream_));
    OCM_CK(cudaMemcpyAsync(e, energy_.p + slot * kNumSlots, sizeof(e), cudaMemcpyDeviceToHost, stream_));
    OCM_CK(cudaMemcpyAsync(&bad, &sys_.p[slot].eval_status, sizeof(int), cudaMemcpyDeviceToHost, stream_));
    OCM_CK(cudaStreamSynchronize(stream_));
    if (forces)
        for (int64_t i = 0; i < S.n; ++i)
            for (int c = 0; c < 3; ++c) forces[3 * i + c] = (double)f[(size_t)c * nmax_ + i];
    if (energies) {
        for (int g = 0; g < 32; ++g) energies[g] = 0.0;
        for (int k = 0; k < kNumSlots; ++k)
            if (S.slot_group[k] >= 0) energies[S.slot_group[k]] += e[k];
    }
    if (bad) throw Error(7, "[error] non-finite or out-of-range force (above 1e9 kJ/mol/nm) in slot " +
                                std::to_string(slot));
}

void BatchEngine::retire(int64_t slot) {
    OCM_CK(cudaSetDevice(device_));
    if (slot < 0 || slot >= max_systems_ || !slots_[slot].used) throw Error(1, "[error] invalid slot");
    sync_steps();
    Slot& S = slots_[slot];
    h_overflow_[slot] = 0;
    h_status_[slot] = 0;
    beads_.release(S.bead_off, S.n);
    blob_.release(S.blob_off, S.blob_size);
    list_alloc_.release(S.list_off, S.list_size);
    S = Slot();
    BatchSys R{};
    sys_host_[slot] = R;
    OCM_CK(cudaMemcpyAsync(sys_.p + slot, &sys_host_[slot], sizeof(BatchSys), cudaMemcpyHostToDevice, stream_));
    OCM_CK(cudaStreamSynchronize(stream_));
}

void BatchEngine::slot_stats(int64_t slot, int32_t* builds, int32_t* capacity) {
    OCM_CK(cudaSetDevice(device_));
    if (slot < 0 || slot >= max_systems_ || !slots_[slot].used) throw Error(1, "[error] invalid slot");
    sync_steps();
    int b = 0;
    OCM_CK(cudaMemcpy(&b, &sys_.p[slot].builds, sizeof(int), cudaMemcpyDeviceToHost));
    *builds = b;
    *capacity = slots_[slot].maxn;
}

// Scatter / gather of many slots' states through one pinned staging buffer
// and one kernel, so a whole ensemble moves host<->device in two copies.
namespace {
// Sets *bad when any of the m values is not finite (|v| <= DBL_MAX is
// false for infinities and NaN).
__global__ void k_check_finite(long long m, const double* __restrict__ v, int* bad) {
    bool ok = true;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < m; k += (long long)gridDim.x * blockDim.x)
        ok = ok && fabs(v[k]) <= DBL_MAX;
    if (!__all_sync(0xffffffffu, ok) && (threadIdx.x & 31) == 0) *bad = 1;
}

// Positions (and velocities) of many slots from the packed staging buffer;
// writes nothing when the check above found a non-finite position.
__global__ void k_scatter_state(int nseg, const long long* __restrict__ seg_bead,
                                const long long* __restrict__ seg_src, const int* __restrict__ seg_n,
                                const double* __restrict__ src, int with_v, double* x, double* y,
                                double* z, float* vx, float* vy, float* vz, long long total,
                                const int* __restrict__ bad) {
    const int g = blockIdx.y;
    if (g >= nseg || *bad) return;
    const int n = seg_n[g];
    const long long b0 = seg_bead[g], s0 = seg_src[g];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const double* p = src + 3 * (s0 + k);
        x[b0 + k] = p[0];
        y[b0 + k] = p[1];
        z[b0 + k] = p[2];
        if (with_v) {
            const double* q = src + 3 * total + 3 * (s0 + k);
            vx[b0 + k] = (float)q[0];
            vy[b0 + k] = (float)q[1];
            vz[b0 + k] = (float)q[2];
        }
    }
}
__global__ void k_gather_pos(int nseg, const long long* __restrict__ seg_bead,
                             const long long* __restrict__ seg_dst, const int* __restrict__ seg_n,
                             const double* x, const double* y, const double* z, double* __restrict__ dst) {
    const int g = blockIdx.y;
    if (g >= nseg) return;
    const int n = seg_n[g];
    const long long b0 = seg_bead[g], d0 = seg_dst[g];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        double* p = dst + 3 * (d0 + k);
        p[0] = x[b0 + k];
        p[1] = y[b0 + k];
        p[2] = z[b0 + k];
    }
}

// Scratch of ocm_batch_get_positions_many_noalloc: file-scope device arrays,
// so that read-out never allocates device memory.  Their addresses are taken
// once per device (noalloc_scratch).  Nothing in them needs to start at
// zero: each call writes the segment table and every staged value it copies
// back.  All batches of one device share them.
constexpr int kNoAllocMaxBeads = 131072;  // 3 MiB of staged positions
constexpr int kNoAllocMaxSlots = 2048;
static __device__ __align__(256) double g_noalloc_stage[3 * kNoAllocMaxBeads];
static __device__ __align__(256) long long g_noalloc_bead[kNoAllocMaxSlots];
static __device__ __align__(256) long long g_noalloc_dst[kNoAllocMaxSlots];
static __device__ __align__(256) int g_noalloc_n[kNoAllocMaxSlots];
}  // namespace

// Segment table of a many-slot copy (each slot's bead offset in the state
// arrays, its offset in the packed host buffer, its bead count), uploaded
// only when it differs from the last one (a loop over the same slots reuses
// it).  The copies are ordered on the engine's stream after any kernel that
// still reads the old table; the host vectors are staged before they
// return.
void BatchEngine::upload_segments(int64_t n, const std::vector<long long>& bead,
                                  const std::vector<long long>& off, const std::vector<int>& cnt) {
    if ((int64_t)seg_n_.n < n) {
        seg_bead_.alloc(n);
        seg_off_.alloc(n);
        seg_n_.alloc(n);
        seg_cnt_h_.clear();
    }
    if (seg_cnt_h_ == cnt && seg_off_h_ == off && seg_bead_h_ == bead) return;
    // on the engine's stream, ahead of the kernel that reads the table
    OCM_CK(cudaMemcpyAsync(seg_bead_.p, bead.data(), n * sizeof(long long), cudaMemcpyHostToDevice, stream_));
    OCM_CK(cudaMemcpyAsync(seg_off_.p, off.data(), n * sizeof(long long), cudaMemcpyHostToDevice, stream_));
    OCM_CK(cudaMemcpyAsync(seg_n_.p, cnt.data(), n * sizeof(int), cudaMemcpyHostToDevice, stream_));
    seg_bead_h_ = bead;
    seg_off_h_ = off;
    seg_cnt_h_ = cnt;
}

void BatchEngine::set_positions_many(int64_t n, const int64_t* slots, const double* xyz,
                                     const double* v) {
    OCM_CK(cudaSetDevice(device_));
    if (n <= 0) return;
    std::vector<long long> bead(n), src(n);
    std::vector<int> cnt(n);
    long long total = 0;
    for (int64_t k = 0; k < n; ++k) {
        const int64_t sl = slots[k];
        if (sl < 0 || sl >= max_systems_ || !slots_[sl].used) throw Error(1, "[error] invalid slot");
        bead[k] = slots_[sl].bead_off;
        src[k] = total;
        cnt[k] = (int)slots_[sl].n;
        total += slots_[sl].n;
    }
    // every step below is ordered on the engine's stream; the positions are
    // checked on the device and written only when all are finite
    upload_segments(n, bead, src, cnt);
    if ((int64_t)stage_.n < (v ? 6 : 3) * total) stage_.alloc((v ? 6 : 3) * total);
    DevBuf<long long>& db = seg_bead_;
    DevBuf<long long>& ds = seg_off_;
    DevBuf<int>& dn = seg_n_;
    DevBuf<double>& buf = stage_;
    cudaStream_t s = stream_;
    OCM_CK(cudaMemcpyAsync(buf.p, xyz, 3 * total * sizeof(double), cudaMemcpyHostToDevice, s));
    if (v) OCM_CK(cudaMemcpyAsync(buf.p + 3 * total, v, 3 * total * sizeof(double), cudaMemcpyHostToDevice, s));
    OCM_CK(cudaMemsetAsync(check_.p, 0, sizeof(int), s));
    k_check_finite<<<(unsigned)std::min<long long>(4 * num_sms_, (3 * total + 255) / 256), 256, 0, s>>>(
        3 * total, buf.p, check_.p);
    const dim3 grid(8, (unsigned)n);
    k_scatter_state<<<grid, 128, 0, s>>>((int)n, db.p, ds.p, dn.p, buf.p, v ? 1 : 0, x_.p, y_.p, z_.p,
                                         vx_.p, vy_.p, vz_.p, total, check_.p);
    OCM_CK(cudaGetLastError());
    OCM_CK(cudaMemcpyAsync(h_check_, check_.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    OCM_CK(cudaStreamSynchronize(s));
    if (*h_check_) throw Error(7, "[error] non-finite position");
}

void BatchEngine::get_positions_many(int64_t n, const int64_t* slots, double* xyz) {
    OCM_CK(cudaSetDevice(device_));
    if (n <= 0) return;
    std::vector<long long> bead(n), dst(n);
    std::vector<int> cnt(n);
    long long total = 0;
    for (int64_t k = 0; k < n; ++k) {
        const int64_t sl = slots[k];
        if (sl < 0 || sl >= max_systems_ || !slots_[sl].used) throw Error(1, "[error] invalid slot");
        bead[k] = slots_[sl].bead_off;
        dst[k] = total;
        cnt[k] = (int)slots_[sl].n;
        total += slots_[sl].n;
    }
    upload_segments(n, bead, dst, cnt);
    if ((int64_t)stage_.n < 3 * total) stage_.alloc(3 * total);
    DevBuf<long long>& db = seg_bead_;
    DevBuf<long long>& dd = seg_off_;
    DevBuf<int>& dn = seg_n_;
    DevBuf<double>& buf = stage_;
    cudaStream_t s = stream_;
    const dim3 grid(8, (unsigned)n);
    k_gather_pos<<<grid, 128, 0, s>>>((int)n, db.p, dd.p, dn.p, x_.p, y_.p, z_.p, buf.p);
    OCM_CK(cudaGetLastError());
    OCM_CK(cudaMemcpyAsync(xyz, buf.p, 3 * total * sizeof(double), cudaMemcpyDeviceToHost, s));
    OCM_CK(cudaStreamSynchronize(s));
}

namespace {
struct NoAllocScratch {
    double* stage = nullptr;
    long long* bead = nullptr;
    long long* dst = nullptr;
    int* n = nullptr;
};

// Device addresses of the no-alloc scratch for `device`, taken with that
// device current on first use and cached (the one set-up step).
NoAllocScratch noalloc_scratch(int device) {
    static std::mutex mu;
    static std::map<int, NoAllocScratch> cache;
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(device);
    if (it != cache.end()) return it->second;
    NoAllocScratch sc;
    OCM_CK(cudaGetSymbolAddress(reinterpret_cast<void**>(&sc.stage), g_noalloc_stage));
    OCM_CK(cudaGetSymbolAddress(reinterpret_cast<void**>(&sc.bead), g_noalloc_bead));
    OCM_CK(cudaGetSymbolAddress(reinterpret_cast<void**>(&sc.dst), g_noalloc_dst));
    OCM_CK(cudaGetSymbolAddress(reinterpret_cast<void**>(&sc.n), g_noalloc_n));
    cache.emplace(device, sc);
    return sc;
}
}  // namespace

void BatchEngine::get_positions_many_noalloc(int64_t n, const int64_t* slots, double* xyz) {
    OCM_CK(cudaSetDevice(device_));
    if (n <= 0) return;
    if (n > kNoAllocMaxSlots)
        throw Error(1, "[error] ocm_batch_get_positions_many_noalloc reads at most " +
                           std::to_string(kNoAllocMaxSlots) + " slots per call (asked for " +
                           std::to_string(n) + "); use ocm_batch_get_positions_many");
    // segment table in per-thread host storage: no heap allocation per call
    thread_local long long h_bead[kNoAllocMaxSlots], h_dst[kNoAllocMaxSlots];
    thread_local int h_n[kNoAllocMaxSlots];
    long long total = 0;
    for (int64_t k = 0; k < n; ++k) {
        const int64_t sl = slots[k];
        if (sl < 0 || sl >= max_systems_ || !slots_[sl].used) throw Error(1, "[error] invalid slot");
        h_bead[k] = slots_[sl].bead_off;
        h_dst[k] = total;
        h_n[k] = (int)slots_[sl].n;
        total += slots_[sl].n;
    }
    if (total > kNoAllocMaxBeads)
        throw Error(1, "[error] ocm_batch_get_positions_many_noalloc reads at most " +
                           std::to_string(kNoAllocMaxBeads) + " beads per call (asked for " +
                           std::to_string(total) + "); use ocm_batch_get_positions_many");
    const NoAllocScratch sc = noalloc_scratch(device_);
    cudaStream_t s = stream_;
    OCM_CK(cudaStreamSynchronize(s));
    OCM_CK(cudaMemcpyAsync(sc.bead, h_bead, n * sizeof(long long), cudaMemcpyHostToDevice, s));
    OCM_CK(cudaMemcpyAsync(sc.dst, h_dst, n * sizeof(long long), cudaMemcpyHostToDevice, s));
    OCM_CK(cudaMemcpyAsync(sc.n, h_n, n * sizeof(int), cudaMemcpyHostToDevice, s));
    const dim3 grid(8, (unsigned)n);
    k_gather_pos<<<grid, 128, 0, s>>>((int)n, sc.bead, sc.dst, sc.n, x_.p, y_.p, z_.p, sc.stage);
    OCM_CK(cudaGetLastError());
    OCM_CK(cudaMemcpyAsync(xyz, sc.stage, 3 * total * sizeof(double), cudaMemcpyDeviceToHost, s));
    OCM_CK(cudaStreamSynchronize(s));
}

void BatchEngine::active(int64_t* n_active, int64_t* beads) {
    int64_t a = 0, b = 0;
    for (const auto& s : slots_)
        if (s.used) {
            ++a;
            b += s.n;
        }
    *n_active = a;
    *beads = b;
}

}  // namespace ocm
