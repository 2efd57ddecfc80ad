// batch_engine.cu - persistent shared-memory kernel for many independent
// systems (the batched ensemble and the serving loop).
//
// One CTA per SM (or more, by occupancy) pulls systems from a work queue
// ordered by decreasing cost.  A claimed system is loaded into shared
// memory (FP64 master positions, FP32 positions and parameters, velocities,
// 64-bit fixed-point force accumulators) and advanced for the whole chunk
// without touching global memory except for L2-resident static parameters:
//   tiles:    every 32x32 cluster pair (I <= J) whose bounding boxes lie
//             within the largest cutoff, recomputed every step - no
//             neighbour list and no skin;
//   bonded:   bonds, Go contacts, FLA, FLD;
//   update:   Langevin step per bead, fused with zeroing the accumulators
//             and recomputing each cluster's bounding box.
// Two __syncthreads per step.  Results depend only on (system, seed, step):
// a system gives the same trajectory alone or in any mix.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
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

__host__ __device__ __forceinline__ int pair_split(int n) {
    int S = 1;
    while (S < kMaxSplit && n * S * 2 <= kSplitUnits) S <<= 1;
    return S;
}

struct BatchArgs {
    BatchSys* sys;
    const int32_t* order;
    int n_order;
    int* head;
    double *x, *y, *z;
    float *vx, *vy, *vz;
    const unsigned char* blob;
    int k;
    int nmax;
    double* energy;              // [slot][kNumSlots]
    unsigned long long* forces;  // eval output [3][nmax]
    uint16_t* lists;             // neighbour-list arena
    uint32_t slots_enabled;
    size_t smem_bytes;           // dynamic shared memory of the launch
};

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

// 64-bit fixed-point force accumulator in shared memory, kept as separate
// low and high 32-bit words ([3][nmax] each).  An addition adds the low word
// with a 32-bit atomic, takes the carry from the returned old value and adds
// high + carry: the final 64-bit value is exact and independent of the order
// of the additions, and two 32-bit shared atomics cost far less than one
// 64-bit shared atomic.
struct FixedAcc {
    uint32_t* lo;
    uint32_t* hi;
};

__device__ __forceinline__ void facc_add(const FixedAcc& F, int idx, float f) {
    const unsigned long long v = to_fixed(f);
    const uint32_t l = (uint32_t)v;
    const uint32_t old = atomicAdd(&F.lo[idx], l);
    const uint32_t h = (uint32_t)(v >> 32) + (old + l < old ? 1u : 0u);
    if (h) atomicAdd(&F.hi[idx], h);
}

__device__ __forceinline__ long long facc_get(const FixedAcc& F, int idx) {
    return (long long)(((unsigned long long)F.hi[idx] << 32) | F.lo[idx]);
}

__device__ __forceinline__ void facc_zero(const FixedAcc& F, int idx) {
    F.lo[idx] = 0u;
    F.hi[idx] = 0u;
}

__device__ __forceinline__ void sadd(const FixedAcc& F, int nmax, int b, float3 f) {
    facc_add(F, b, f.x);
    facc_add(F, nmax + b, f.y);
    facc_add(F, 2 * nmax + b, f.z);
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

template <int TERMS, bool LABELS, bool ENERGY>
__device__ __forceinline__ void batch_tile(int I, int J, int mslot, const uint32_t* __restrict__ masks,
                                           const float4* sx, const float4* sp0, const float4* sp1,
                                           const uint32_t* slab, const FixedAcc& sF, int nmax,
                                           const PairConsts& pc, uint32_t excl_all, int lane,
                                           float* eacc) {
    const int ki = I * 32 + lane, kj = J * 32 + lane;
    const float4 xi = sx[ki];
    const float4 p0i = sp0[ki];
    const float4 p1i = (TERMS & kTermLJA) ? sp1[ki] : make_float4(0.f, 0.f, 0.f, 0.f);
    const uint32_t labi = LABELS ? slab[ki] : 0u;
    float4 xj = sx[kj];
    float4 p0j = sp0[kj];
    float4 p1j = (TERMS & kTermLJA) ? sp1[kj] : make_float4(0.f, 0.f, 0.f, 0.f);
    uint32_t labj = LABELS ? slab[kj] : 0u;
    uint32_t mw[4] = {0u, 0u, 0u, 0u};
    if (mslot >= 0) {
#pragma unroll
        for (int term = 0; term < 4; ++term)
            if (TERMS & (1 << term)) mw[term] = masks[(size_t)mslot * 128 + term * 32 + lane];
    }
    const bool diag = I == J;
    float3 fi = make_float3(0.f, 0.f, 0.f), fj = make_float3(0.f, 0.f, 0.f);
    PairEnergy e;
    e.zero();
    const float3 nobox = make_float3(0.f, 0.f, 0.f);
    for (int r = 0; r < 32; ++r) {
        const bool do_pair = !diag || (r > 0 && (r < 16 || (r == 16 && lane < 16)));
        if (do_pair) {
            const float3 d = separation<false>(xi, xj, nobox, nobox);
            const float r2 = norm2(d);
            if (r2 < pc.list_rc2) {
                uint32_t ex = excl_all;
#pragma unroll
                for (int term = 0; term < 4; ++term)
                    if (TERMS & (1 << term)) ex |= ((mw[term] >> r) & 1u) << term;
                if (LABELS) {
#pragma unroll
                    for (int term = 0; term < 4; ++term)
                        if ((TERMS & (1 << term)) && (pc.uses_labels & (1 << term)) &&
                            !labels_allow(labi, labj, term, pc.allow[term]))
                            ex |= 1u << term;
                }
                const float s = pair_scalar<TERMS, ENERGY>(r2, p0i, p0j, p1i, p1j, ex, pc, e);
                fi.x -= s * d.x;
                fi.y -= s * d.y;
                fi.z -= s * d.z;
                fj.x += s * d.x;
                fj.y += s * d.y;
                fj.z += s * d.z;
            }
        }
        const int src = (lane + 1) & 31;
        xj.x = __shfl_sync(kFull, xj.x, src);
        xj.y = __shfl_sync(kFull, xj.y, src);
        xj.z = __shfl_sync(kFull, xj.z, src);
        if (TERMS & kTermEXV) p0j.x = __shfl_sync(kFull, p0j.x, src);
        if (TERMS & kTermDH) p0j.y = __shfl_sync(kFull, p0j.y, src);
        if (TERMS & kTermLJR) {
            p0j.z = __shfl_sync(kFull, p0j.z, src);
            p0j.w = __shfl_sync(kFull, p0j.w, src);
        }
        if (TERMS & kTermLJA) {
            p1j.x = __shfl_sync(kFull, p1j.x, src);
            p1j.y = __shfl_sync(kFull, p1j.y, src);
        }
        if (LABELS) labj = __shfl_sync(kFull, labj, src);
        fj.x = __shfl_sync(kFull, fj.x, src);
        fj.y = __shfl_sync(kFull, fj.y, src);
        fj.z = __shfl_sync(kFull, fj.z, src);
    }
    sadd(sF, nmax, ki, fi);
    sadd(sF, nmax, kj, fj);
    if (ENERGY) {
        eacc[kSlotEXV] += e.exv;
        eacc[kSlotDH] += e.dh;
        eacc[kSlotLJR] += e.ljr;
        eacc[kSlotLJA] += e.lja;
    }
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

__device__ __forceinline__ bool bbox_close(float4 ci, float4 hi, float4 cj, float4 hj, float cut2) {
    const float gx = fmaxf(0.f, fabsf(cj.x - ci.x) - hi.x - hj.x);
    const float gy = fmaxf(0.f, fabsf(cj.y - ci.y) - hi.y - hj.y);
    const float gz = fmaxf(0.f, fabsf(cj.z - ci.z) - hi.z - hj.z);
    return gx * gx + gy * gy + gz * gz < cut2;
}

// Neighbour list of every bead of the claimed system, built by one thread
// per bead: all j != i whose FP32 r^2 (canonical form) is below cut2, in
// increasing j, so the list and every FP32 sum over it are deterministic.
// Entry = j | (excluded-term bits << 11); pairs excluded for every present
// term are dropped.  Entry k of bead i lives in shared memory at
// slist[k * npad + i] for k < cap_s and in global memory at
// glist[k * npad + i] for cap_s <= k < maxn.  Sets *overflow when a list
// exceeds maxn.
template <bool LABELS>
__device__ __forceinline__ void build_lists(int n, int nt, int npad, int maxn, int cap_s, float cut2,
                                            const float4* sx, const uint32_t* slab,
                                            const float4* bc, const float4* bh,
                                            const int32_t* __restrict__ ex_start,
                                            const int32_t* __restrict__ ex,
                                            const PairConsts& pc, uint16_t* slist,
                                            uint16_t* __restrict__ glist, uint16_t* scnt,
                                            float* sref, int nmax, int tid, int threads,
                                            int S, uint16_t* sseg, int* overflow) {
    const float3 nobox = make_float3(0.f, 0.f, 0.f);
    const uint32_t present = (uint32_t)pc.terms;
    for (int i = tid; i < n; i += threads) {
        const float4 xi = sx[i];
        const uint32_t labi = LABELS ? slab[i] : 0u;
        int cnt = 0;
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
                while (ej < j) {
                    ++ep;
                    ej = ep < e1 ? (ex[ep] & 0xFFFFFF) : 0x7FFFFFFF;
                }
                uint32_t bits = ej == j ? ((uint32_t)ex[ep] >> 24) : 0u;
                if (LABELS) {
                    const uint32_t labj = slab[j];
#pragma unroll
                    for (int term = 0; term < 4; ++term)
                        if ((pc.uses_labels & (1 << term)) && !labels_allow(labi, labj, term, pc.allow[term]))
                            bits |= 1u << term;
                }
                if ((bits & present) == present) continue;
                while (j >= jb) {
                    sseg[i * S + s_next] = (uint16_t)min(cnt, maxn);
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
    }
}

// Pair forces on bead i from list entries [k0, cnt), four entries per
// iteration so their loads and arithmetic overlap.  One accumulator, in list
// (= increasing j) order: entries outside the cutoff contribute nothing, so
// the FP32 sum does not depend on when the list was built.
template <int TERMS, bool ENERGY>
__device__ __forceinline__ float3 list_forces(int i, int k0, int cnt, int cap_s, int npad,
                                              const uint16_t* slist,
                                              const uint16_t* __restrict__ glist,
                                              const float4* sx, const float4* sp0,
                                              const float4* sp1, uint32_t excl_all,
                                              const PairConsts& pc, PairEnergy& e) {
    const float3 nobox = make_float3(0.f, 0.f, 0.f);
    const float4 xi = sx[i];
    const float4 p0i = sp0[i];
    const float4 p1i = (TERMS & kTermLJA) ? sp1[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    float3 fa = make_float3(0.f, 0.f, 0.f);
    for (int k = k0; k < cnt; k += 4) {
        uint32_t ent[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int kk = k + u;
            ent[u] = kk < cnt ? (kk < cap_s ? (uint32_t)slist[kk * npad + i]
                                            : (uint32_t)glist[(size_t)kk * npad + i])
                              : 0xFFFFFFFFu;
        }
        float4 xj[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) xj[u] = sx[ent[u] != 0xFFFFFFFFu ? (int)(ent[u] & 2047u) : i];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (ent[u] == 0xFFFFFFFFu) continue;
            const int j = (int)(ent[u] & 2047u);
            const float3 d = separation<false>(xi, xj[u], nobox, nobox);
            const float r2 = norm2(d);
            if (r2 < pc.list_rc2) {
                const float4 p0j = sp0[j];
                const float4 p1j = (TERMS & kTermLJA) ? sp1[j] : make_float4(0.f, 0.f, 0.f, 0.f);
                const float s = pair_scalar<TERMS, ENERGY>(r2, p0i, p0j, p1i, p1j,
                                                           (ent[u] >> 11) | excl_all, pc, e);
                fa.x -= s * d.x;
                fa.y -= s * d.y;
                fa.z -= s * d.z;
            }
        }
    }
    return fa;
}

constexpr int kMaxBeadsPerThread = 8;  // 2048 beads / 256 threads

template <int THREADS, int TERMS, bool LABELS, bool ENERGY, bool INTEGRATE>
__global__ void __launch_bounds__(THREADS, 1) k_batch(BatchArgs a) {
    constexpr int NW = THREADS / 32;
    constexpr int BPT = (32 * kMaxClusters + THREADS - 1) / THREADS;  // beads per thread
    extern __shared__ __align__(16) unsigned char smem[];
    const int nmax = a.nmax;  // stride of the global force output
    __shared__ int s_claim;
    __shared__ int s_move[2];
    __shared__ int s_overflow;
    __shared__ double s_energy[kNumSlots];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const float nan = __int_as_float(0x7fc00000);

    while (true) {
        if (tid == 0) {
            s_claim = atomicAdd(a.head, 1);
            s_move[0] = 0;
            s_move[1] = 0;
            s_overflow = 0;
        }
        if (ENERGY && tid < kNumSlots) s_energy[tid] = 0.0;
        __syncthreads();
        const int q = s_claim;
        if (q >= a.n_order) break;
        const int slot = a.order[q];
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
        // parts in sxl; x = hi + lo carries ~48 significant bits.
        const int ns = npad;
        const FixedAcc sF{reinterpret_cast<uint32_t*>(smem), reinterpret_cast<uint32_t*>(smem) + 3 * ns};
        float4* sx = reinterpret_cast<float4*>(smem + 24 * (size_t)ns);
        float4* sp0 = reinterpret_cast<float4*>(smem + 40 * (size_t)ns);
        float* sxl = reinterpret_cast<float*>(smem + 56 * (size_t)ns);
        float* sv = reinterpret_cast<float*>(smem + 68 * (size_t)ns);
        float* sim = reinterpret_cast<float*>(smem + 80 * (size_t)ns);
        float* sref = reinterpret_cast<float*>(smem + 84 * (size_t)ns);
        uint16_t* scnt = reinterpret_cast<uint16_t*>(smem + 96 * (size_t)ns);
        size_t off = 98 * (size_t)ns;
        float4* sp1 = nullptr;
        uint32_t* slab = nullptr;
        if ((TERMS & kTermLJA) || LABELS) {
            sp1 = reinterpret_cast<float4*>(smem + off);
            slab = reinterpret_cast<uint32_t*>(smem + off + 16 * (size_t)ns);
            off += 20 * (size_t)ns;
        }
        float4* bc = reinterpret_cast<float4*>(smem + off);
        float4* bh = bc + nt;
        off += 32 * (size_t)nt;
        uint16_t* sseg = reinterpret_cast<uint16_t*>(smem + off);
        off += 2 * kMaxUnits;
        // bonded records and tables: staged in shared memory when they fit,
        // read from the blob otherwise
        const unsigned char* gbonded = blob + R.off_bonded;
        const bool bonded_smem = off + (size_t)R.bonded_bytes <= a.smem_bytes;
        unsigned char* sbonded = smem + off;
        if (bonded_smem) off += (size_t)R.bonded_bytes;
        const unsigned char* bsrc = bonded_smem ? sbonded : gbonded;
        const float4* bpar = reinterpret_cast<const float4*>(bsrc + R.rb_p);
        const uint32_t* bij = reinterpret_cast<const uint32_t*>(bsrc + R.rb_ij);
        const uint2* aij = reinterpret_cast<const uint2*>(bsrc + R.ra_ij);
        const float* ak = reinterpret_cast<const float*>(bsrc + R.ra_k);
        const uint4* drec = reinterpret_cast<const uint4*>(bsrc + R.rd);
        const float2* gdp = reinterpret_cast<const float2*>(bsrc + R.rgd);
        const FlaTable* fla = reinterpret_cast<const FlaTable*>(bsrc + R.rfla);
        const FldTable* fld = reinterpret_cast<const FldTable*>(bsrc + R.rfld);
        uint16_t* slist = reinterpret_cast<uint16_t*>(smem + off);
        const size_t list_bytes = a.smem_bytes > off ? a.smem_bytes - off : 0;
        const int32_t* tmask = reinterpret_cast<const int32_t*>(blob + R.off_tmask);
        const uint32_t* masks = reinterpret_cast<const uint32_t*>(blob + R.off_masks);
        const int32_t* ex_start = reinterpret_cast<const int32_t*>(blob + R.off_ex_start);
        const int32_t* exl = reinterpret_cast<const int32_t*>(blob + R.off_ex);
        uint16_t* glist = a.lists + R.list_off;
        const int maxn = R.maxn;
        // entries per bead kept in shared memory (multiple of 4)
        const int cap_s = min(maxn, (int)(list_bytes / (2 * (size_t)npad)) & ~3);
        const int n_bonds = R.n_bonds, n_angles = R.n_angles, n_dih = R.n_dih;
        const int S = pair_split(n);
        const unsigned long long step0 = R.steps_done;
        int K = 1;
        if (INTEGRATE) {
            const unsigned long long left = R.steps_target > step0 ? R.steps_target - step0 : 0ull;
            K = (int)min((unsigned long long)a.k, left);
        }
        const uint32_t slots_en = INTEGRATE ? 0xffffffffu : a.slots_enabled;
        uint32_t excl_all = 0u;
        if (!(slots_en & (1u << kSlotEXV))) excl_all |= kTermEXV;
        if (!(slots_en & (1u << kSlotDH))) excl_all |= kTermDH;
        if (!(slots_en & (1u << kSlotLJR))) excl_all |= kTermLJR;
        if (!(slots_en & (1u << kSlotLJA))) excl_all |= kTermLJA;
        const bool pairs_on = (pc.terms & ~excl_all) != 0;

        // ---- load ----
        for (int b = tid; b < npad; b += THREADS) {
            facc_zero(sF, b);
            facc_zero(sF, ns + b);
            facc_zero(sF, 2 * ns + b);
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
            for (int q = tid; q < R.bonded_bytes / 16; q += THREADS) dst[q] = src[q];
        }
        __syncthreads();
        for (int I = warp; I < nt; I += NW) cluster_bbox(I, n, sx, bc, bh, lane);
        __syncthreads();

        // list cutoff = largest pair cutoff + skin; tiles use the cutoff alone
        const float rc = sqrtf(pc.list_rc2);
        const float lcut = (rc + R.skin) * 1.0001f;
        const float lcut2 = lcut * lcut;
        const float tcut = rc * 1.0001f + 1e-4f;
        const float tcut2 = tcut * tcut;
        const float half_skin2 = 0.25f * R.skin * R.skin;
        bool use_tiles = false;
        bool need_build = pairs_on;
        int builds = 0;
        float eacc[kNumSlots];
#pragma unroll
        for (int k = 0; k < kNumSlots; ++k) eacc[k] = 0.f;

        for (int st = 0; st < K; ++st) {
            if (need_build && !use_tiles) {
                build_lists<LABELS>(n, nt, npad, maxn, cap_s, lcut2, sx, slab, bc, bh, ex_start, exl,
                                    pc, slist, glist, scnt, sref, ns, tid, THREADS, S, sseg,
                                    &s_overflow);
                ++builds;
                __syncthreads();
                use_tiles = s_overflow != 0;
            }
            const unsigned long long step = step0 + (unsigned long long)st;
            // Langevin noise for this thread's beads, drawn before the force
            // work so its latency overlaps the pair loop.
            float3 noise[BPT];
            if (INTEGRATE) {
#pragma unroll
                for (int c = 0; c < BPT; ++c) {
                    const int b = tid + c * THREADS;
                    noise[c] = b < n ? gaussian3(lc.seed, lc.stream, (uint32_t)b, step, kPurposeLangevin)
                                     : make_float3(0.f, 0.f, 0.f);
                }
            }
            // ---- pair terms ----
            if (pairs_on && !use_tiles && S > 1) {
                // (bead, j-range) units u = i * S + s, 32 per warp; the S
                // partial sums of a bead meet in a fixed butterfly
                for (int base = warp * 32; base < n * S; base += THREADS) {
                    const int u = base + lane;
                    const int i = u / S, sr = u & (S - 1);
                    float3 fi = make_float3(0.f, 0.f, 0.f);
                    PairEnergy e;
                    e.zero();
                    if (i < n) {
                        const int k0 = sseg[u];
                        const int k1 = sr == S - 1 ? (int)scnt[i] : (int)sseg[u + 1];
                        fi = list_forces<TERMS, ENERGY>(i, k0, k1, cap_s, npad, slist, glist, sx, sp0,
                                                        sp1, excl_all, pc, e);
                    }
                    for (int o = 1; o < S; o <<= 1) {
                        fi.x += __shfl_xor_sync(kFull, fi.x, o);
                        fi.y += __shfl_xor_sync(kFull, fi.y, o);
                        fi.z += __shfl_xor_sync(kFull, fi.z, o);
                    }
                    if (i < n && sr == 0) sadd(sF, ns, i, fi);
                    if (ENERGY) {
                        eacc[kSlotEXV] += 0.5f * e.exv;
                        eacc[kSlotDH] += 0.5f * e.dh;
                        eacc[kSlotLJR] += 0.5f * e.ljr;
                        eacc[kSlotLJA] += 0.5f * e.lja;
                    }
                }
            } else if (pairs_on && !use_tiles) {
#pragma unroll
                for (int c = 0; c < BPT; ++c) {
                    const int i = tid + c * THREADS;
                    if (i >= n) break;
                    PairEnergy e;
                    e.zero();
                    const float3 fi = list_forces<TERMS, ENERGY>(i, 0, scnt[i], cap_s, npad, slist, glist,
                                                                 sx, sp0, sp1, excl_all, pc, e);
                    sadd(sF, ns, i, fi);
                    if (ENERGY) {
                        // every pair appears in both lists
                        eacc[kSlotEXV] += 0.5f * e.exv;
                        eacc[kSlotDH] += 0.5f * e.dh;
                        eacc[kSlotLJR] += 0.5f * e.ljr;
                        eacc[kSlotLJA] += 0.5f * e.lja;
                    }
                }
            } else if (pairs_on) {
                for (int t = warp; t < R.n_tiles; t += NW) {
                    int J = (int)((sqrtf(8.f * (float)t + 1.f) - 1.f) * 0.5f);
                    while ((J + 1) * (J + 2) / 2 <= t) ++J;
                    while (J * (J + 1) / 2 > t) --J;
                    const int I = t - J * (J + 1) / 2;
                    if (!bbox_close(bc[I], bh[I], bc[J], bh[J], tcut2)) continue;
                    batch_tile<TERMS, LABELS, ENERGY>(I, J, tmask[t], masks, sx, sp0, sp1, slab, sF,
                                                      ns, pc, excl_all, lane, eacc);
                }
            }
            // ---- bonded: one flattened loop over dihedrals | angles |
            // bonds, so the costliest terms spread over all threads ----
            {
                const int n_ad = n_dih + n_angles, n_all = n_ad + n_bonds;
                const bool fld_on = (slots_en & (1u << kSlotFLD)) != 0;
                const bool fla_on = (slots_en & (1u << kSlotFLA)) != 0;
                const bool gd_on = (slots_en & (1u << kSlotGD)) != 0;
                for (int t = tid; t < n_all; t += THREADS) {
                    if (t < n_dih) {
                        const uint4 qd = drec[t];
                        const bool gauss = (qd.x >> 31) != 0;
                        if (!(gauss ? gd_on : fld_on)) continue;
                        const int qi = qd.x & 0xFFFF, qj = (qd.x >> 16) & 0x7FFF, qk = qd.y & 0xFFFF,
                                  ql = qd.y >> 16;
                        const float3 F = ffsep(sx, sxl, ns, qj, qi);
                        const float3 G = ffsep(sx, sxl, ns, qk, qj);
                        const float3 H = ffsep(sx, sxl, ns, qk, ql);
                        float3 f1, f2, f3, f4;
                        float en;
                        if (gauss) {
                            const float2 gp = gdp[qd.z];
                            gauss_dihedral_forces(F, G, H, __uint_as_float(qd.w), gp.x, gp.y, f1, f2, f3, f4,
                                                  en);
                        } else {
                            fld_forces(F, G, H, __uint_as_float(qd.w), fld[qd.z], f1, f2, f3, f4, en);
                        }
                        sadd(sF, ns, qi, f1);
                        sadd(sF, ns, qj, f2);
                        sadd(sF, ns, qk, f3);
                        sadd(sF, ns, ql, f4);
                        if (ENERGY) eacc[gauss ? kSlotGD : kSlotFLD] += en;
                    } else if (t < n_ad) {
                        if (!fla_on) continue;
                        const int b = t - n_dih;
                        const uint2 g = aij[b];
                        const int gi = g.x & 0xFFFF, gj = g.x >> 16, gk = g.y & 0xFFFF;
                        const float3 u = ffsep(sx, sxl, ns, gj, gi);
                        const float3 v = ffsep(sx, sxl, ns, gj, gk);
                        float3 f1, f3;
                        float en;
                        fla_forces(u, v, ak[b], fla[g.y >> 16], f1, f3, en);
                        sadd(sF, ns, gi, f1);
                        sadd(sF, ns, gk, f3);
                        sadd(sF, ns, gj, make_float3(-f1.x - f3.x, -f1.y - f3.y, -f1.z - f3.z));
                        if (ENERGY) eacc[kSlotFLA] += en;
                    } else {
                        const int b = t - n_ad;
                        const uint32_t ij = bij[b];
                        const int kind = (int)(ij >> 30);
                        const int sl = bond_slot(kind);
                        if (!(slots_en & (1u << sl))) continue;
                        const int bi = ij & 0xFFFF, bj = (ij >> 16) & 0x3FFF;
                        const float4 bp = bpar[b];
                        float3 dh, dl;
                        ff_sep(sx[bi], lo3(sxl, ns, bi), sx[bj], lo3(sxl, ns, bj), dh, dl);
                        const float3 d = make_float3(dh.x + dl.x, dh.y + dl.y, dh.z + dl.z);
                        const float delta = ff_bond_delta(dh, dl, bp.z, bp.w);
                        float en;
                        const float sc = bond_scalar(kind, norm2(d), delta, bp.x, bp.y, bp.z, en);
                        sadd(sF, ns, bi, make_float3(-sc * d.x, -sc * d.y, -sc * d.z));
                        sadd(sF, ns, bj, make_float3(sc * d.x, sc * d.y, sc * d.z));
                        if (ENERGY) eacc[sl] += en;
                    }
                }
            }
            __syncthreads();
            if (!INTEGRATE) break;
            // ---- Langevin update, bounding boxes, displacement check ----
            // Bead b = tid + c * THREADS is cluster b / 32 handled by this warp.
            const int mv = st & 1;
#pragma unroll
            for (int c = 0; c < BPT; ++c) {
                const int I = warp + c * NW;
                if (I >= nt) break;
                const int b = I * 32 + lane;
                bool moved = false;
                if (b < n) {
                    const float fx = fixed_to_float(facc_get(sF, b));
                    const float fy = fixed_to_float(facc_get(sF, ns + b));
                    const float fz = fixed_to_float(facc_get(sF, 2 * ns + b));
                    facc_zero(sF, b);
                    facc_zero(sF, ns + b);
                    facc_zero(sF, 2 * ns + b);
                    const float im = sim[b];
                    if (im > 0.f) {
                        const float3 g = noise[c];
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
                        const float dx = h.x - sref[b], dy = h.y - sref[ns + b], dz = h.z - sref[2 * ns + b];
                        moved = dx * dx + dy * dy + dz * dz > half_skin2;
                    }
                }
                if (__any_sync(kFull, moved) && lane == 0) atomicOr(&s_move[mv], 1);
                __syncwarp();
                cluster_bbox(I, n, sx, bc, bh, lane);
            }
            __syncthreads();
            need_build = s_move[mv] != 0;
            if (tid == 0) s_move[mv ^ 1] = 0;
        }

        // ---- write back ----
        if (INTEGRATE) {
            for (int b = tid; b < n; b += THREADS) {
                const float4 h = sx[b];
                a.x[boff + b] = (double)h.x + (double)sxl[b];
                a.y[boff + b] = (double)h.y + (double)sxl[ns + b];
                a.z[boff + b] = (double)h.z + (double)sxl[2 * ns + b];
                a.vx[boff + b] = sv[b];
                a.vy[boff + b] = sv[ns + b];
                a.vz[boff + b] = sv[2 * ns + b];
            }
            if (tid == 0) {
                a.sys[slot].steps_done = step0 + (unsigned long long)K;
                a.sys[slot].builds = builds;
                if (s_overflow) a.sys[slot].overflow = 1;
            }
        } else {
            for (int b = tid; b < n; b += THREADS) {
                a.forces[b] = (unsigned long long)facc_get(sF, b);
                a.forces[nmax + b] = (unsigned long long)facc_get(sF, ns + b);
                a.forces[2 * nmax + b] = (unsigned long long)facc_get(sF, 2 * ns + b);
            }
            if (tid == 0 && s_overflow) a.sys[slot].overflow = 1;
        }
        if (ENERGY) {
#pragma unroll
            for (int k = 0; k < kNumSlots; ++k) {
                const double v = warp_sum_d((double)eacc[k]);
                if (lane == 0 && v != 0.0) atomicAdd(&s_energy[k], v);
            }
            __syncthreads();
            if (tid < kNumSlots) a.energy[(size_t)slot * kNumSlots + tid] = s_energy[tid];
        }
        __syncthreads();
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
    int optin = 0, per_sm_smem = 0, dev = 0;
    OCM_CK(cudaGetDevice(&dev));
    OCM_CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    OCM_CK(cudaDeviceGetAttribute(&per_sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    cudaFuncAttributes fa{};
    OCM_CK(cudaFuncGetAttributes(&fa, fn));
    const int max_dyn = optin - (int)fa.sharedSizeBytes;
    OCM_CK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dyn));
    int per_sm = 0;
    OCM_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem));
    if (per_sm < 1) throw Error(6, "[error] batched kernel does not fit on an SM");
    size_t share = (size_t)per_sm_smem / per_sm;
    share = share > 2048 ? share - 2048 : share;  // static + reserved per block
    share = std::min<size_t>(share, (size_t)max_dyn);
    if (want > 0) share = std::min(share, want);
    share = std::max(share, smem) & ~(size_t)15;
    a.smem_bytes = share;
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

struct BlobLayout {
    int64_t size = 0;
    int off_p0, off_p1, off_lab, off_invm, off_tmask, off_masks, off_ex_start, off_ex;
    int off_bonded, bonded_bytes, rb_p, rb_ij, ra_ij, ra_k, rd, rgd, rfla, rfld;
    int n_tiles, n_masks;
};

BlobLayout blob_layout(const CompiledSystem& c, int n_masks) {
    BlobLayout L{};
    const int64_t n = c.n;
    const int nt = (int)((n + 31) / 32);
    L.n_tiles = nt * (nt + 1) / 2;
    L.n_masks = n_masks;
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
    // indices (uint2) | angle k (f32) | dihedral records (uint4) | FLA | FLD
    L.off_bonded = (int)o;
    const int64_t nb = (int64_t)c.bonds.size(), na = (int64_t)c.angles.size(),
                  nd = (int64_t)c.dihedrals.size();
    L.rb_p = take(16 * nb) - L.off_bonded;
    L.rb_ij = take(4 * nb) - L.off_bonded;
    L.ra_ij = take(8 * na) - L.off_bonded;
    L.ra_k = take(4 * na) - L.off_bonded;
    L.rd = take(16 * nd) - L.off_bonded;
    int64_t ngd = 0;
    for (const auto& t : c.dihedrals) ngd += t.kind == kDihGauss ? 1 : 0;
    L.rgd = take(8 * ngd) - L.off_bonded;
    L.rfla = take((int64_t)sizeof(FlaTable) * c.fla.size()) - L.off_bonded;
    L.rfld = take((int64_t)sizeof(FldTable) * c.fld.size()) - L.off_bonded;
    L.bonded_bytes = (int)(o - L.off_bonded);
    L.off_tmask = take(4 * (int64_t)L.n_tiles);
    L.off_masks = take(4 * 128 * (int64_t)n_masks);
    L.off_ex_start = take(4 * (n + 1));
    L.off_ex = take(4 * (int64_t)c.ex_j.size());
    L.size = align_up(o, 256);
    return L;
}

// Exclusion masks in chain order: tile index t = J(J+1)/2 + I (I <= J).
void build_masks(const CompiledSystem& c, std::vector<int32_t>& tmask, std::vector<uint32_t>& masks) {
    const int nt = (int)((c.n + 31) / 32);
    tmask.assign(nt * (nt + 1) / 2, -1);
    masks.clear();
    for (int64_t i = 0; i < c.n; ++i) {
        for (int32_t e = c.ex_start[i]; e < c.ex_start[i + 1]; ++e) {
            const int64_t j = c.ex_j[e];
            if (j <= i) continue;
            const int I = (int)(i >> 5), J = (int)(j >> 5);
            const int t = J * (J + 1) / 2 + I;
            if (tmask[t] < 0) {
                tmask[t] = (int32_t)(masks.size() / 128);
                masks.resize(masks.size() + 128, 0u);
            }
            uint32_t* w = &masks[(size_t)tmask[t] * 128];
            const int li = (int)(i & 31), lj = (int)(j & 31);
            for (int term = 0; term < kNumPairTerms; ++term) {
                if (!(c.ex_bits[e] & (1 << term))) continue;
                w[term * 32 + li] |= 1u << ((lj - li) & 31);
                if (I == J) w[term * 32 + lj] |= 1u << ((li - lj) & 31);
            }
        }
    }
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
    sys_.alloc(max_systems);
    OCM_CK(cudaMemset(sys_.p, 0, sizeof(BatchSys) * max_systems));
    order_.alloc(max_systems);
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
    if (stream_) cudaStreamDestroy(stream_);
    if (copy_stream_) cudaStreamDestroy(copy_stream_);
}

size_t BatchEngine::smem_bytes(int nmax, bool general) const {
    return (size_t)nmax * (general ? 118 : 98) + 2 * kMaxClusters * sizeof(float4) + 2 * kMaxUnits;
}

int64_t BatchEngine::footprint(const SystemDesc& d) {
    CompiledSystem c = compile_system(d);
    std::vector<int32_t> tm;
    std::vector<uint32_t> mk;
    build_masks(c, tm, mk);
    const BlobLayout L = blob_layout(c, (int)(mk.size() / 128));
    return L.size + c.n * (3 * 8 + 3 * 4) + (int64_t)sizeof(BatchSys);
}

void BatchEngine::set_list_smem(int kib) {
    if (kib < -1 || kib > 228) throw Error(1, "[error] list shared memory must be -1 or 0..228 KiB");
    list_smem_kib_ = kib;
}

void BatchEngine::set_threads(int threads) {
    if (threads != 256 && threads != 512 && threads != 1024)
        throw Error(1, "[error] threads per CTA must be 256, 512 or 1024");
    threads_ = threads;
}

int64_t BatchEngine::admit(const SystemDesc& d, const double* pos, const double* vel, double T,
                           double friction, double dt, int32_t seed, int64_t n_steps) {
    OCM_CK(cudaSetDevice(device_));
    if (n_steps < 0) throw Error(1, "[error] negative step count");
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
    std::vector<int32_t> tmask;
    std::vector<uint32_t> masks;
    build_masks(c, tmask, masks);
    const BlobLayout L = blob_layout(c, (int)(masks.size() / 128));
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
        std::vector<float4> bp(c.bonds.size());
        std::vector<uint32_t> bij(c.bonds.size());
        for (size_t b = 0; b < c.bonds.size(); ++b) {
            const BondTerm& t = c.bonds[b];
            bp[b] = make_float4(t.p0, t.p1, t.r0sq_hi, t.r0sq_lo);
            bij[b] = (uint32_t)t.i | ((uint32_t)t.j << 16) | ((uint32_t)t.kind << 30);
        }
        std::vector<uint2> aij(c.angles.size());
        std::vector<float> ak(c.angles.size());
        for (size_t b = 0; b < c.angles.size(); ++b) {
            const AngleTerm& t = c.angles[b];
            aij[b] = make_uint2((uint32_t)t.i | ((uint32_t)t.j << 16), (uint32_t)t.k | ((uint32_t)t.table << 16));
            ak[b] = t.kk;
        }
        // dihedral record: FLD table index, or (bit 31 of .x set) the index
        // of the Gaussian dihedral's (theta0, 1 / (2 sigma^2))
        std::vector<uint4> dr(c.dihedrals.size());
        std::vector<float2> gd;
        for (size_t b = 0; b < c.dihedrals.size(); ++b) {
            const DihedralTerm& t = c.dihedrals[b];
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
    }
    put(L.off_tmask, tmask.data(), 4 * tmask.size());
    put(L.off_masks, masks.data(), 4 * masks.size());
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
    R.n_tiles = L.n_tiles;
    R.n_bonds = (int)c.bonds.size();
    R.n_angles = (int)c.angles.size();
    R.n_dih = (int)c.dihedrals.size();
    R.n_masks = L.n_masks;
    R.off_p0 = L.off_p0; R.off_p1 = L.off_p1; R.off_lab = L.off_lab; R.off_invm = L.off_invm;
    R.off_bonded = L.off_bonded; R.bonded_bytes = L.bonded_bytes;
    R.rb_p = L.rb_p; R.rb_ij = L.rb_ij; R.ra_ij = L.ra_ij; R.ra_k = L.ra_k; R.rd = L.rd; R.rgd = L.rgd;
    R.rfla = L.rfla; R.rfld = L.rfld;
    R.off_tmask = L.off_tmask; R.off_masks = L.off_masks;
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
    R.steps_done = 0;
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
    S.steps_done = 0;
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
                         cudaStream_t s) {
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
    OCM_CK(cudaMemsetAsync(head_.p, 0, sizeof(int32_t), s));
    BatchArgs a{};
    a.sys = sys_.p;
    a.order = order_.p;
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
    std::vector<int32_t> order;
    for (int64_t s = 0; s < max_systems_; ++s)
        if (slots_[s].used && slots_[s].steps_done < slots_[s].steps_target) order.push_back((int32_t)s);
    std::stable_sort(order.begin(), order.end(),
                     [&](int32_t a, int32_t b) { return slots_[a].cost > slots_[b].cost; });
    grow_lists();
    OCM_CK(cudaStreamWaitEvent(stream_, ev_copy_, 0));
    OCM_CK(cudaEventRecord(ev0_, stream_));
    if (!order.empty()) launch(true, false, k, order, stream_);
    OCM_CK(cudaEventRecord(ev1_, stream_));
    OCM_CK(cudaMemcpy2DAsync(h_overflow_, sizeof(int), &sys_.p[0].overflow, sizeof(BatchSys),
                             sizeof(int), max_systems_, cudaMemcpyDeviceToHost, stream_));
    ran_ = true;
    for (int32_t q : order)
        slots_[q].steps_done = std::min<uint64_t>(slots_[q].steps_target, slots_[q].steps_done + k);
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

void BatchEngine::sync_steps() { OCM_CK(cudaStreamSynchronize(stream_)); }

// A list that overflowed made its system fall back to the tile sweep for
// the rest of that chunk (same results, more work); give it more room now.
void BatchEngine::grow_lists() {
    if (!ran_) return;
    OCM_CK(cudaStreamSynchronize(stream_));
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
        if (!slots_[s].used || slots_[s].steps_done < slots_[s].steps_target) continue;
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
    std::vector<unsigned long long> f(3 * nmax_);
    double e[kNumSlots];
    OCM_CK(cudaMemcpyAsync(f.data(), forces_.p, 3 * nmax_ * sizeof(unsigned long long),
                           cudaMemcpyDeviceToHost, stream_));
    OCM_CK(cudaMemcpyAsync(e, energy_.p + slot * kNumSlots, sizeof(e), cudaMemcpyDeviceToHost, stream_));
    OCM_CK(cudaStreamSynchronize(stream_));
    if (forces)
        for (int64_t i = 0; i < S.n; ++i)
            for (int c = 0; c < 3; ++c)
                forces[3 * i + c] = (double)(long long)f[(size_t)c * nmax_ + i] * kFixedInv;
    if (energies) {
        for (int g = 0; g < 32; ++g) energies[g] = 0.0;
        for (int k = 0; k < kNumSlots; ++k)
            if (S.slot_group[k] >= 0) energies[S.slot_group[k]] += e[k];
    }
}

void BatchEngine::retire(int64_t slot) {
    OCM_CK(cudaSetDevice(device_));
    if (slot < 0 || slot >= max_systems_ || !slots_[slot].used) throw Error(1, "[error] invalid slot");
    sync_steps();
    Slot& S = slots_[slot];
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
__global__ void k_scatter_state(int nseg, const long long* __restrict__ seg_bead,
                                const long long* __restrict__ seg_src, const int* __restrict__ seg_n,
                                const double* __restrict__ src, int with_v, double* x, double* y,
                                double* z, float* vx, float* vy, float* vz, long long total) {
    const int g = blockIdx.y;
    if (g >= nseg) return;
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
    for (long long k = 0; k < 3 * total; ++k)
        if (!std::isfinite(xyz[k])) throw Error(7, "[error] non-finite position");
    OCM_CK(cudaStreamSynchronize(stream_));
    if ((int64_t)seg_n_.n < n) {
        seg_bead_.alloc(n);
        seg_off_.alloc(n);
        seg_n_.alloc(n);
    }
    if ((int64_t)stage_.n < (v ? 6 : 3) * total) stage_.alloc((v ? 6 : 3) * total);
    DevBuf<long long>& db = seg_bead_;
    DevBuf<long long>& ds = seg_off_;
    DevBuf<int>& dn = seg_n_;
    DevBuf<double>& buf = stage_;
    cudaStream_t s = stream_;
    OCM_CK(cudaMemcpyAsync(db.p, bead.data(), n * sizeof(long long), cudaMemcpyHostToDevice, s));
    OCM_CK(cudaMemcpyAsync(ds.p, src.data(), n * sizeof(long long), cudaMemcpyHostToDevice, s));
    OCM_CK(cudaMemcpyAsync(dn.p, cnt.data(), n * sizeof(int), cudaMemcpyHostToDevice, s));
    OCM_CK(cudaMemcpyAsync(buf.p, xyz, 3 * total * sizeof(double), cudaMemcpyHostToDevice, s));
    if (v) OCM_CK(cudaMemcpyAsync(buf.p + 3 * total, v, 3 * total * sizeof(double), cudaMemcpyHostToDevice, s));
    const dim3 grid(8, (unsigned)n);
    k_scatter_state<<<grid, 128, 0, s>>>((int)n, db.p, ds.p, dn.p, buf.p, v ? 1 : 0, x_.p, y_.p, z_.p,
                                         vx_.p, vy_.p, vz_.p, total);
    OCM_CK(cudaGetLastError());
    OCM_CK(cudaStreamSynchronize(s));
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
    OCM_CK(cudaStreamSynchronize(stream_));
    if ((int64_t)seg_n_.n < n) {
        seg_bead_.alloc(n);
        seg_off_.alloc(n);
        seg_n_.alloc(n);
    }
    if ((int64_t)stage_.n < 3 * total) stage_.alloc(3 * total);
    DevBuf<long long>& db = seg_bead_;
    DevBuf<long long>& dd = seg_off_;
    DevBuf<int>& dn = seg_n_;
    DevBuf<double>& buf = stage_;
    cudaStream_t s = stream_;
    OCM_CK(cudaMemcpyAsync(db.p, bead.data(), n * sizeof(long long), cudaMemcpyHostToDevice, s));
    OCM_CK(cudaMemcpyAsync(dd.p, dst.data(), n * sizeof(long long), cudaMemcpyHostToDevice, s));
    OCM_CK(cudaMemcpyAsync(dn.p, cnt.data(), n * sizeof(int), cudaMemcpyHostToDevice, s));
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
