// plain_engine.cu - the plain single-system path.
//
// Per step: one fused force kernel (cluster-pair tiles for the pair terms,
// segments for bonds / Go / Gaussian / capped-Go contacts, angles,
// dihedrals and, when Debye-Hueckel reaches further than the other pair
// terms, its per-bead charged rows, all in one grid) and one Langevin kernel
// that also zeroes the fixed-point force buffer.  Every `rebuild_interval`
// steps the cluster layout and the lists are rebuilt:
//   cell keys (x-y columns, z slices; periodic systems) -> counting sort
//   with in-cell ranks -> gather into cluster order with anchored offsets
//   -> bounding boxes and anchors -> candidate tiles (count / scan / fill)
//   -> exact pruning -> compaction with per-tile anchor shifts ->
//   exclusion masks; charged-bead cells -> charged rows.
// A chunk of steps (rebuild + steps) is captured once into a CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "batch_engine.hpp"
#include "device_math.cuh"
#include "engine.hpp"

namespace ocm {

void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess)
        throw Error(2, std::string("[error] CUDA: ") + what + ": " + cudaGetErrorString(e));
}

namespace {

constexpr int kForceThreads = 128;
constexpr int kWarpsPerForceBlock = kForceThreads / 32;
constexpr int kTilesPerChunk = 1;  // measured on the 20k-bead slab: 1 -> 65, 2 -> 71, 4 -> 76 us per step
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ float4 shfl4(float4 v, int src) {
    v.x = __shfl_sync(kFull, v.x, src);
    v.y = __shfl_sync(kFull, v.y, src);
    v.z = __shfl_sync(kFull, v.z, src);
    return v;
}

// ---------------------------------------------------------------------------
// Cluster-anchored coordinates.  Each cluster has an anchor, the FP32 centre
// of its bounding box at the last list build; a bead is stored as its offset
// from the anchor, taken in FP64 from the master position and rounded once
// to FP32 (|offset| of a nm or two, so about 1e-7 nm of rounding instead of
// the ~1e-5 nm of an FP32 coordinate 150 nm from the origin).  A pair's
// separation is (o_j - o_i) + (a_J - a_I), the anchor shift formed exactly in
// FP64 and rounded once per tile.  All steps are individually rounded so a
// host enumeration reproduces r^2 bit for bit.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double wrap_coord(double x, double L, double invL) {
    const double k = floor(__dmul_rn(x, invL));
    return __dsub_rn(x, __dmul_rn(k, L));
}

// w - a in FP64, rounded once to FP32; when periodic and |w - a| > L/2,
// first the minimum image e - L rint(e / L).
__device__ __forceinline__ float anchor_offset(double w, float a, double L, double iL, int periodic) {
    double e = __dsub_rn(w, (double)a);
    if (periodic && fabs(e) > 0.5 * L) e = __dsub_rn(e, __dmul_rn(L, rint(__dmul_rn(e, iL))));
    return __double2float_rn(e);
}

__device__ __forceinline__ float3 anchor_shift(float4 ai, float4 aj, const BoxD& b) {
    return make_float3(anchor_offset((double)aj.x, ai.x, b.L[0], b.iL[0], b.periodic),
                       anchor_offset((double)aj.y, ai.y, b.L[1], b.iL[1], b.periodic),
                       anchor_offset((double)aj.z, ai.z, b.L[2], b.iL[2], b.periodic));
}

__device__ __forceinline__ float3 anchored_sep(float4 oi, float4 oj, float3 A) {
    return make_float3(__fadd_rn(__fsub_rn(oj.x, oi.x), A.x), __fadd_rn(__fsub_rn(oj.y, oi.y), A.y),
                       __fadd_rn(__fsub_rn(oj.z, oi.z), A.z));
}

// The FP32 minimum-image step of the canonical separation.
__device__ __forceinline__ float3 min_image(float3 d, const float3& box, const float3& inv_box) {
    d.x = __fmaf_rn(-box.x, rintf(__fmul_rn(d.x, inv_box.x)), d.x);
    d.y = __fmaf_rn(-box.y, rintf(__fmul_rn(d.y, inv_box.y)), d.y);
    d.z = __fmaf_rn(-box.z, rintf(__fmul_rn(d.z, inv_box.z)), d.z);
    return d;
}

// x_j - x_i from float-float positions (hi = FP32 box-frame coordinate, lo =
// its FP64 remainder): fl(fl(hj - hi) + fl(lj - li)), then the minimum image.
template <bool PERIODIC>
__device__ __forceinline__ float3 ff_separation(float4 hi_i, float4 lo_i, float4 hi_j, float4 lo_j,
                                                const float3& box, const float3& inv_box) {
    float3 d = make_float3(__fadd_rn(__fsub_rn(hi_j.x, hi_i.x), __fsub_rn(lo_j.x, lo_i.x)),
                           __fadd_rn(__fsub_rn(hi_j.y, hi_i.y), __fsub_rn(lo_j.y, lo_i.y)),
                           __fadd_rn(__fsub_rn(hi_j.z, hi_i.z), __fsub_rn(lo_j.z, lo_i.z)));
    if (PERIODIC) d = min_image(d, box, inv_box);
    return d;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

// ---------------------------------------------------------------------------
// Rebuild kernels
// ---------------------------------------------------------------------------

// Exclusive scan of m ints into out[0..m] (out[m] = total) by one block of
// 1024 threads: each of the 32 warps owns a contiguous segment and reads it
// 32 consecutive values at a time (coalesced) - once for the segment total,
// once more to write the prefixes with a shuffle scan.
__device__ __forceinline__ void block_scan(int m, const int32_t* __restrict__ in, int32_t* __restrict__ out) {
    __shared__ int32_t wsum[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int per = (m + 31) / 32;
    const int b = w * per, e = min(m, b + per);
    int32_t s = 0;
    for (int i = b + lane; i < e; i += 32) s += in[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(kFull, s, o);
    if (lane == 0) wsum[w] = s;
    __syncthreads();
    if (w == 0) {  // inclusive scan of the 32 segment totals
        int32_t v = wsum[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t u = __shfl_up_sync(kFull, v, o);
            if (lane >= o) v += u;
        }
        wsum[lane] = v;
    }
    __syncthreads();
    int32_t run = w > 0 ? wsum[w - 1] : 0;
    for (int i0 = b; i0 < e; i0 += 32) {  // warp-uniform bounds
        const int i = i0 + lane;
        const int32_t v = i < e ? in[i] : 0;
        int32_t x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t u = __shfl_up_sync(kFull, x, o);
            if (lane >= o) x += u;
        }
        if (i < e) out[i] = run + x - v;
        run += __shfl_sync(kFull, x, 31);
    }
    if (threadIdx.x == 0) out[m] = wsum[31];
}

__global__ void __launch_bounds__(1024) k_scan(int m, const int32_t* __restrict__ in,
                                               int32_t* __restrict__ out) {
    block_scan(m, in, out);
}

// Two independent scans in one launch, one block each.
__global__ void __launch_bounds__(1024) k_scan2(int m0, const int32_t* __restrict__ in0, int32_t* __restrict__ out0,
                                                int m1, const int32_t* __restrict__ in1, int32_t* __restrict__ out1) {
    if (blockIdx.x == 0) block_scan(m0, in0, out0);
    else block_scan(m1, in1, out1);
}

// Cell keys of the beads (columns) and, in the same launch, of the charged
// beads (their own grid): threads [0, n) and [n, n + m).
__global__ void k_keys_both(int n, const float4* __restrict__ xq, int nx, int ny, int nz, float3 box,
                            int32_t* __restrict__ key, int32_t* __restrict__ count, int m,
                            const int32_t* __restrict__ cidx, int cnx, int cny, int cnz,
                            int32_t* __restrict__ ckey, int32_t* __restrict__ ccount) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) {
        const float4 p = xq[t];
        const int cx = min(nx - 1, max(0, (int)(p.x * ((float)nx / box.x))));
        const int cy = min(ny - 1, max(0, (int)(p.y * ((float)ny / box.y))));
        const int cz = min(nz - 1, max(0, (int)(p.z * ((float)nz / box.z))));
        const int k = (cy * nx + cx) * nz + cz;
        key[t] = k;
        atomicAdd(&count[k], 1);
    } else if (t < n + m) {
        const int c = t - n;
        const float4 p = xq[cidx[c]];
        const int cx = min(cnx - 1, max(0, (int)(p.x * ((float)cnx / box.x))));
        const int cy = min(cny - 1, max(0, (int)(p.y * ((float)cny / box.y))));
        const int cz = min(cnz - 1, max(0, (int)(p.z * ((float)cnz / box.z))));
        const int k = (cz * cny + cy) * cnx + cx;
        ckey[c] = k;
        atomicAdd(&ccount[k], 1);
    }
}

// Start slot of every column (exclusive scan of its bead count rounded up to
// whole clusters), one block of 1024 threads.
__global__ void __launch_bounds__(1024) k_col_scan(int ncols, int nz, const int32_t* __restrict__ cell_start,
                                                   int32_t* __restrict__ col_start) {
    __shared__ int32_t part[1024];
    const int t = threadIdx.x;
    const int per = (ncols + 1023) / 1024;
    const int b = t * per, e = min(ncols, b + per);
    auto slots = [&](int c) { return (cell_start[(c + 1) * nz] - cell_start[c * nz] + 31) & ~31; };
    int32_t s = 0;
    for (int c = b; c < e; ++c) s += slots(c);
    part[t] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const int32_t v = t >= o ? part[t - o] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    int32_t run = part[t] - s;
    for (int c = b; c < e; ++c) {
        col_start[c] = run;
        run += slots(c);
    }
    if (t == 1023) col_start[ncols] = part[1023];
}


// Cluster order: columns one after another (each padded to whole clusters),
// inside a column the z slices bottom-up, inside a slice ascending index.
// One thread per bead ranks it among its cell's members by index, so the
// order does not depend on the atomic timing of the scatter.
__global__ void k_bucket_rank(int n, int nz, const int32_t* __restrict__ key,
                              const int32_t* __restrict__ start, const int32_t* __restrict__ col_start,
                              const int32_t* __restrict__ bucket, int32_t* __restrict__ perm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = key[i], col = c / nz;
    const int b = start[c], e = start[c + 1];
    int rank = 0;
    for (int q = b; q < e; ++q) rank += bucket[q] < i;
    perm[col_start[col] + (b - start[col * nz]) + rank] = i;
}

// Cluster order: anchors, anchored offsets and the parameters of every slot.
__global__ void k_gather_sorted(int np, const int32_t* __restrict__ perm,
                                const float4* __restrict__ xq, const double* __restrict__ x,
                                const double* __restrict__ y, const double* __restrict__ z, BoxD bd,
                                const float4* __restrict__ p0,
                                const float4* __restrict__ p1, const uint32_t* __restrict__ lab,
                                int32_t* __restrict__ slot, float4* __restrict__ xs,
                                float4* __restrict__ anc,
                                float4* __restrict__ p0s, float4* __restrict__ p1s,
                                uint32_t* __restrict__ labs, float4* __restrict__ ref) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= np) return;
    const int o = perm[k];
    const int o0 = perm[k & ~31];
    const float nan = __int_as_float(0x7fc00000);
    const float4 a = o0 >= 0 ? xq[o0] : make_float4(nan, nan, nan, 0.f);
    if ((k & 31) == 0) anc[k >> 5] = a;
    if (o >= 0) {
        slot[o] = k;
        const float4 p = xq[o];
        double w[3] = {x[o], y[o], z[o]};
        if (bd.periodic)
            for (int c = 0; c < 3; ++c) w[c] = wrap_coord(w[c], bd.L[c], bd.iL[c]);
        xs[k] = make_float4(anchor_offset(w[0], a.x, bd.L[0], bd.iL[0], bd.periodic),
                            anchor_offset(w[1], a.y, bd.L[1], bd.iL[1], bd.periodic),
                            anchor_offset(w[2], a.z, bd.L[2], bd.iL[2], bd.periodic), 0.f);
        ref[o] = p;
        p0s[k] = p0[o];
        p1s[k] = p1[o];
        labs[k] = lab[o];
    } else {
        xs[k] = make_float4(nan, nan, nan, 0.f);
        p0s[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        p1s[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        labs[k] = 0xffffffffu;
    }
}

// Bounding box of each cluster from the offsets to its first bead: centre
// (FP32 box frame, the cluster's anchor from here on) and half widths (w < 0
// marks a cluster of padding slots only).
__global__ void k_bbox(int nc, const float4* __restrict__ xs, const float4* __restrict__ anc,
                       const int32_t* __restrict__ perm, float4* __restrict__ bc,
                       float4* __restrict__ bh) {
    const int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (I >= nc) return;
    const bool valid = perm[I * 32 + lane] >= 0;
    const float4 o = xs[I * 32 + lane];
    const float4 o0 = make_float4(__shfl_sync(kFull, o.x, 0), __shfl_sync(kFull, o.y, 0),
                                  __shfl_sync(kFull, o.z, 0), 0.f);
    const float4 d = valid ? o : o0;  // slot 0 holds a bead whenever any slot does
    float lx = d.x, ly = d.y, lz = d.z, hx = d.x, hy = d.y, hz = d.z;
    const bool any = __ballot_sync(kFull, valid) != 0u;
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
        lx = fminf(lx, __shfl_xor_sync(kFull, lx, s));
        ly = fminf(ly, __shfl_xor_sync(kFull, ly, s));
        lz = fminf(lz, __shfl_xor_sync(kFull, lz, s));
        hx = fmaxf(hx, __shfl_xor_sync(kFull, hx, s));
        hy = fmaxf(hy, __shfl_xor_sync(kFull, hy, s));
        hz = fmaxf(hz, __shfl_xor_sync(kFull, hz, s));
    }
    if (lane == 0) {
        const float4 a = anc[I];
        bc[I] = make_float4(__fadd_rn(a.x, 0.5f * __fadd_rn(lx, hx)), __fadd_rn(a.y, 0.5f * __fadd_rn(ly, hy)),
                            __fadd_rn(a.z, 0.5f * __fadd_rn(lz, hz)), 0.f);
        bh[I] = make_float4(0.5f * (hx - lx), 0.5f * (hy - ly), 0.5f * (hz - lz), any ? 0.f : -1.f);
    }
}

template <bool PERIODIC>
__device__ __forceinline__ bool boxes_close(float4 ci, float4 hi, float4 cj, float4 hj,
                                            float3 box, float3 inv_box, float cut, float cut2) {
    float dx = cj.x - ci.x, dy = cj.y - ci.y, dz = cj.z - ci.z;
    float gx, gy, gz;
    if (PERIODIC) {
        dx -= box.x * rintf(dx * inv_box.x);
        dy -= box.y * rintf(dy * inv_box.y);
        dz -= box.z * rintf(dz * inv_box.z);
        // Boxes this large relative to the period may meet through another
        // image: treat that dimension as overlapping.
        gx = (hi.x + hj.x + cut >= 0.5f * box.x) ? 0.f : fmaxf(0.f, fabsf(dx) - hi.x - hj.x);
        gy = (hi.y + hj.y + cut >= 0.5f * box.y) ? 0.f : fmaxf(0.f, fabsf(dy) - hi.y - hj.y);
        gz = (hi.z + hj.z + cut >= 0.5f * box.z) ? 0.f : fmaxf(0.f, fabsf(dz) - hi.z - hj.z);
    } else {
        gx = fmaxf(0.f, fabsf(dx) - hi.x - hj.x);
        gy = fmaxf(0.f, fabsf(dy) - hi.y - hj.y);
        gz = fmaxf(0.f, fabsf(dz) - hi.z - hj.z);
    }
    return gx * gx + gy * gy + gz * gz < cut2;
}

// Offsets again, now from the bounding-box centres (the anchors), and the
// largest |offset| per axis of every cluster.  One warp per cluster.
__global__ void k_reanchor(int np, const int32_t* __restrict__ perm, const double* __restrict__ x,
                           const double* __restrict__ y, const double* __restrict__ z, BoxD bd,
                           const float4* __restrict__ bc, float4* __restrict__ anc, float4* __restrict__ xs,
                           float4* __restrict__ ext) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= np) return;  // np is a multiple of 32: whole warps
    const int o = perm[k];
    const float4 a = bc[k >> 5];
    float ex = 0.f, ey = 0.f, ez = 0.f;
    if (o >= 0) {
        double w[3] = {x[o], y[o], z[o]};
        if (bd.periodic)
            for (int c = 0; c < 3; ++c) w[c] = wrap_coord(w[c], bd.L[c], bd.iL[c]);
        const float4 v = make_float4(anchor_offset(w[0], a.x, bd.L[0], bd.iL[0], bd.periodic),
                                     anchor_offset(w[1], a.y, bd.L[1], bd.iL[1], bd.periodic),
                                     anchor_offset(w[2], a.z, bd.L[2], bd.iL[2], bd.periodic), 0.f);
        xs[k] = v;
        ex = fabsf(v.x);
        ey = fabsf(v.y);
        ez = fabsf(v.z);
    }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
        ex = fmaxf(ex, __shfl_xor_sync(kFull, ex, s));
        ey = fmaxf(ey, __shfl_xor_sync(kFull, ey, s));
        ez = fmaxf(ez, __shfl_xor_sync(kFull, ez, s));
    }
    if ((k & 31) == 0) {
        anc[k >> 5] = a;
        ext[k >> 5] = make_float4(ex, ey, ez, 0.f);
    }
}

template <bool PERIODIC, bool FILL>
__global__ void k_tiles(int nc, const float4* __restrict__ bc, const float4* __restrict__ bh,
                        float3 box, float3 inv_box, float cut, float cut2,
                        int32_t* __restrict__ count, const int32_t* __restrict__ start,
                        int32_t* __restrict__ tile_i, int32_t* __restrict__ tile_j, int cap,
                        int32_t* __restrict__ flags) {
    const int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (I >= nc) return;
    if (FILL && start[nc] > cap) {
        if (I == 0 && lane == 0) atomicOr(flags, ListFlags::kTileOverflow);
        return;
    }
    const float4 ci = bc[I], hi = bh[I];
    int pos = FILL ? start[I] : 0;
    for (int J0 = I; J0 < nc && hi.w >= 0.f; J0 += 32) {
        const int J = J0 + lane;
        bool ok = false;
        if (J < nc) {
            const float4 hj = bh[J];
            ok = hj.w >= 0.f && boxes_close<PERIODIC>(ci, hi, bc[J], hj, box, inv_box, cut, cut2);
        }
        const unsigned b = __ballot_sync(kFull, ok);
        if (FILL && ok) {
            const int at = pos + __popc(b & ((1u << lane) - 1u));
            tile_i[at] = I;
            tile_j[at] = J;
        }
        pos += __popc(b);
    }
    if (!FILL && lane == 0) count[I] = pos;
}

// Pruning of the candidate tiles (bounding boxes within range): one warp
// per candidate tile, lanes on the row cluster's beads, the column cluster's
// beads broadcast one at a time; a tile is kept if any pair is within range
// (the diagonal tile always).  kept_count[I] counts the kept tiles of row I.
template <bool PERIODIC>
__global__ void k_prune(int nc, const float4* __restrict__ xs, const float4* __restrict__ anc,
                        const int32_t* __restrict__ raw_start,
                        const int32_t* __restrict__ raw_i, const int32_t* __restrict__ raw_j, int cap,
                        float3 box, float3 inv_box, float cut2, uint8_t* __restrict__ keep_flag,
                        int32_t* __restrict__ kept_count) {
    const int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int total = raw_start[nc];
    if (t >= total || total > cap) return;  // warp-uniform
    const int I = raw_i[t], J = raw_j[t];
    bool keep = I == J;
    if (!keep) {
        const float4 xi = xs[I * 32 + lane];
        // FP32 anchor shift: the pruning cutoff carries the skin and a
        // 1e-4 nm margin, far above this rounding
        const float4 ai = anc[I], aj = anc[J];
        float3 A = make_float3(__fsub_rn(aj.x, ai.x), __fsub_rn(aj.y, ai.y), __fsub_rn(aj.z, ai.z));
        if (PERIODIC) A = min_image(A, box, inv_box);
        for (int k = 0; k < 32 && !keep; ++k) {
            float3 d = anchored_sep(xi, xs[J * 32 + k], A);
            if (PERIODIC) d = min_image(d, box, inv_box);
            const float r2 = norm2(d);
            keep = __ballot_sync(kFull, r2 < cut2) != 0u;
        }
    }
    if (lane == 0) {
        keep_flag[t] = keep ? 1 : 0;
        if (keep) atomicAdd(&kept_count[I], 1);
    }
}

// Kept tiles of every row, in their order, into the final list (exclusion
// masks cleared): one warp per row, compacted by ballot.  Each tile also
// gets its anchor shift a_J - a_I and, in w, whether its pairs need the FP32
// minimum image: not when |shift| + both clusters' largest offsets + pad
// (the offsets' growth allowance until the next build) stays under half the
// box, where the minimum image leaves every separation unchanged anyway.
__global__ void k_compact_tiles(int nc, const int32_t* __restrict__ raw_start, const int32_t* __restrict__ raw_j,
                                const uint8_t* __restrict__ keep_flag, int cap, const int32_t* __restrict__ start,
                                const float4* __restrict__ anc, const float4* __restrict__ ext, BoxD bd,
                                float3 box, float pad, int32_t* __restrict__ tile_i, int32_t* __restrict__ tile_j,
                                int32_t* __restrict__ tile_mask, float4* __restrict__ tile_shift) {
    const int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (I >= nc || raw_start[nc] > cap) return;
    const int r0 = raw_start[I], r1 = raw_start[I + 1];
    const float4 ai = anc[I], ei = ext[I];
    int at = start[I];
    for (int q0 = r0; q0 < r1; q0 += 32) {
        const int q = q0 + lane;
        const bool keep = q < r1 && keep_flag[q];
        const unsigned b = __ballot_sync(kFull, keep);
        if (keep) {
            const int k = at + __popc(b & ((1u << lane) - 1u));
            const int J = raw_j[q];
            tile_i[k] = I;
            tile_j[k] = J;
            tile_mask[k] = -1;
            const float3 A = anchor_shift(ai, anc[J], bd);
            const float4 ej = ext[J];
            const bool wrap = bd.periodic && (fabsf(A.x) + ei.x + ej.x + pad >= 0.5f * box.x ||
                                              fabsf(A.y) + ei.y + ej.y + pad >= 0.5f * box.y ||
                                              fabsf(A.z) + ei.z + ej.z + pad >= 0.5f * box.z);
            tile_shift[k] = make_float4(A.x, A.y, A.z, wrap ? 1.f : 0.f);
        }
        at += __popc(b);
    }
}

__device__ __forceinline__ int find_tile(const int32_t* __restrict__ start,
                                         const int32_t* __restrict__ tile_j, int a, int b) {
    int lo = start[a], hi = start[a + 1] - 1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const int v = tile_j[mid];
        if (v == b) return mid;
        if (v < b) lo = mid + 1;
        else hi = mid - 1;
    }
    return -1;
}

template <bool FILLBITS>
__global__ void k_excl(int nnz, int nc, int tile_cap, const int32_t* __restrict__ ex_i, const int32_t* __restrict__ ex_j,
                       const uint8_t* __restrict__ ex_bits, const int32_t* __restrict__ slot,
                       const int32_t* __restrict__ start, const int32_t* __restrict__ tile_j,
                       int32_t* __restrict__ tile_mask, uint32_t* __restrict__ masks,
                       int32_t* __restrict__ mask_count, int mask_cap,
                       int32_t* __restrict__ flags) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nnz) return;
    if (start[nc] > tile_cap) return;  // overflowed list: never read past capacity
    const int i = ex_i[e], j = ex_j[e];
    if (i >= j) return;
    const int si = slot[i], sj = slot[j];
    const int ci = si >> 5, cj = sj >> 5;
    const int a = min(ci, cj), b = max(ci, cj);
    const int t = find_tile(start, tile_j, a, b);
    if (t < 0) return;
    if (!FILLBITS) {
        if (atomicCAS(&tile_mask[t], -1, -2) == -1) {
            const int m = atomicAdd(mask_count, 1);
            if (m >= mask_cap) {
                atomicOr(flags, ListFlags::kMaskOverflow);
                tile_mask[t] = -1;
                return;
            }
            for (int w = 0; w < 128; ++w) masks[(size_t)m * 128 + w] = 0u;
            __threadfence();
            tile_mask[t] = m;
        }
        return;
    }
    const int m = tile_mask[t];
    if (m < 0) return;
    const int bits = ex_bits[e];
    // word (term, i-lane) bit r: pair (i-lane, (i-lane + r) & 31)
    int la, lb;
    if (ci <= cj) {
        la = si & 31;
        lb = sj & 31;
    } else {
        la = sj & 31;
        lb = si & 31;
    }
    for (int term = 0; term < kNumPairTerms; ++term) {
        if (!(bits & (1 << term))) continue;
        atomicOr(&masks[(size_t)m * 128 + term * 32 + la], 1u << ((lb - la) & 31));
        if (ci == cj) atomicOr(&masks[(size_t)m * 128 + term * 32 + lb], 1u << ((la - lb) & 31));
    }
}

// ---------------------------------------------------------------------------
// Charged-pair list (Debye-Hueckel beyond the other terms' cutoffs): a cell
// grid over the charged beads, cells at least (cutoff + skin) wide, and per
// charged bead t a row of every charged partner j != i within range that the
// Debye-Hueckel exclusions keep (both directions of each pair are listed, so
// the force kernel writes only bead i's force and needs no atomics per pair).
// A row's order depends on atomic timing in the cell scatter; the forces do
// not, because each pair's force is rounded to fixed point before it is
// summed.
// ---------------------------------------------------------------------------

// Bucket scatter of the beads and, in the same launch, of the charged
// beads, whose records (position, bead index in w) are grouped by cell so
// the row build reads one contiguous record per candidate: threads [0, n)
// and [n, n + m).
__global__ void k_scatter_both(int n, const int32_t* __restrict__ key, const int32_t* __restrict__ start,
                               int32_t* __restrict__ fill, int32_t* __restrict__ bucket, int m,
                               const int32_t* __restrict__ cidx, const int32_t* __restrict__ ckey,
                               const float4* __restrict__ xq, const int32_t* __restrict__ cstart,
                               int32_t* __restrict__ cfill, float4* __restrict__ sorted) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) {
        const int k = key[t];
        bucket[start[k] + atomicAdd(&fill[k], 1)] = t;
    } else if (t < n + m) {
        const int c = t - n;
        const int k = ckey[c], i = cidx[c];
        const float4 p = xq[i];
        sorted[cstart[k] + atomicAdd(&cfill[k], 1)] = make_float4(p.x, p.y, p.z, __int_as_float(i));
    }
}

// One warp per charged bead: the 27 neighbour cells (the three cells of a
// row along x as one range where they do not wrap), 32 candidates at a time,
// kept partners compacted by ballot.  row_stats[0] is the longest row,
// row_stats[1] the number of row entries.
__global__ void k_chg_rows(int m, const int32_t* __restrict__ idx, const int32_t* __restrict__ key,
                           const float4* __restrict__ xq, int nx, int ny, int nz, float3 box,
                           float3 inv_box, float cut2, const int32_t* __restrict__ start,
                           const float4* __restrict__ sorted, const int32_t* __restrict__ ex_csr,
                           const int32_t* __restrict__ ex_j, const uint8_t* __restrict__ ex_bits,
                           int32_t* __restrict__ rows, int32_t* __restrict__ row_len, int row_cap,
                           int32_t* __restrict__ row_stats, int32_t* flags) {
    const int lane = threadIdx.x & 31;
    const int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (t >= m) return;  // warp-uniform
    const int i = idx[t];
    const float4 xi = xq[i];
    const int k = key[t];
    const int cx = k % nx, cy = (k / nx) % ny, cz = k / (nx * ny);
    const int e0 = ex_csr[i], e1 = ex_csr[i + 1];
    // the row's excluded partners span [ex_lo, ex_hi] (sorted): candidates
    // outside skip the search
    const int ex_lo = e0 < e1 ? ex_j[e0] : 1, ex_hi = e0 < e1 ? ex_j[e1 - 1] : 0;
    int32_t* row = rows + (size_t)t * row_cap;
    int len = 0;
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy) {
            const int r = (((cz + dz + nz) % nz) * ny + (cy + dy + ny) % ny) * nx;
            const bool inner = cx > 0 && cx < nx - 1;
            for (int seg = 0; seg < (inner ? 1 : 3); ++seg) {
                const int q_begin = inner ? start[r + cx - 1] : start[r + (cx + seg - 1 + nx) % nx];
                const int q_end = inner ? start[r + cx + 2] : start[r + (cx + seg - 1 + nx) % nx + 1];
                for (int q0 = q_begin; q0 < q_end; q0 += 32) {
                    const int q = q0 + lane;
                    bool keep = false;
                    int j = 0;
                    if (q < q_end) {
                        const float4 c = sorted[q];
                        j = __float_as_int(c.w);
                        if (j != i) {
                            const float r2 = norm2(separation<true>(xi, c, box, inv_box));
                            keep = r2 < cut2;
                            if (keep && j >= ex_lo && j <= ex_hi) {
                                int lo = e0, hi = e1;  // this row's exclusions, sorted by j
                                while (lo < hi) {
                                    const int mid = (lo + hi) >> 1;
                                    if (ex_j[mid] < j) lo = mid + 1;
                                    else hi = mid;
                                }
                                if (lo < e1 && ex_j[lo] == j && (ex_bits[lo] & kTermDH)) keep = false;
                            }
                        }
                    }
                    const unsigned bal = __ballot_sync(0xffffffffu, keep);
                    if (keep) {
                        const int at = len + __popc(bal & ((1u << lane) - 1u));
                        if (at < row_cap) row[at] = j;
                    }
                    len += __popc(bal);
                }
            }
        }
    if (lane == 0) {
        row_len[t] = len;
        atomicMax(&row_stats[0], len);
        atomicAdd(&row_stats[1], len);
        if (len > row_cap) atomicOr(flags, ListFlags::kChargedOverflow);
    }
}

// Verification: the charged pairs (i < j) of the rows whose FP32 r^2 is
// below the Debye-Hueckel cutoff squared.
__global__ void k_chg_list_pairs(int m, const int32_t* __restrict__ idx, const int32_t* __restrict__ rows,
                                 const int32_t* __restrict__ row_len, int row_cap,
                                 const float4* __restrict__ xq, const float4* __restrict__ xlo, float3 box,
                                 float3 inv_box, float rc2, long long* out, long long out_cap,
                                 unsigned long long* count) {
    const int t = blockIdx.x;
    if (t >= m) return;
    const int i = idx[t];
    const int len = min(row_len[t], row_cap);
    for (int p = threadIdx.x; p < len; p += blockDim.x) {
        const int j = rows[(size_t)t * row_cap + p];
        if (j < i) continue;
        const float r2 = norm2(ff_separation<true>(xq[i], xlo[i], xq[j], xlo[j], box, inv_box));
        if (r2 < rc2) {
            const unsigned long long at = atomicAdd(count, 1ull);
            if ((long long)at < out_cap) {
                out[2 * at] = i;
                out[2 * at + 1] = j;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Fused force kernel
// ---------------------------------------------------------------------------
struct ForceArgs {
    int tile_cap;
    int nc, blocks_tiles, blocks_bonds, blocks_angles, blocks_dih, blocks_chg;
    int n;
    const float4 *xs, *p0s, *p1s;
    const uint32_t* labs;
    const int32_t *perm, *tile_start, *tile_i, *tile_j, *tile_mask;
    const uint32_t* masks;
    const double *x, *y, *z;
    int n_bonds, n_angles, n_dih;
    const BondTerm* bonds;
    const AngleTerm* angles;
    const FlaTable* fla;
    const DihedralTerm* dih;
    const FldTable* fld;
    unsigned long long* F;
    PairConsts pc;
    float3 box, inv_box;
    uint32_t slots_enabled;
    uint32_t excl_all;
    double* energy;
    const float4* tile_shift;  // per tile: anchor shift a_J - a_I, w != 0: minimum image needed
    // charged-pair rows (blocks_chg > 0)
    const float4 *xq, *xlo, *p0;
    const int32_t *chg_idx, *chg_rows, *chg_len;
    int n_chg, chg_row_cap;
    int32_t* flags;
};

// A force of this size (kJ/mol/nm) or more, or a non-finite one, marks a
// blown-up system: the 64-bit accumulators hold |F| < 2^31 at 2^32 units
// per kJ/mol/nm, so sums of such contributions could wrap.
constexpr float kForceLimit = 1.0e9f;

__device__ __forceinline__ bool force_ok(float3 f) {
    return fabsf(f.x) < kForceLimit && fabsf(f.y) < kForceLimit && fabsf(f.z) < kForceLimit;
}

__device__ __forceinline__ void add_force(const ForceArgs& a, int i, float3 f) {
    if (!force_ok(f)) atomicOr(a.flags, ListFlags::kBlownUp);
    fixed_add(&a.F[i], f.x);
    fixed_add(&a.F[a.n + i], f.y);
    fixed_add(&a.F[2 * a.n + i], f.z);
}

__device__ __forceinline__ float3 bonded_sep(const ForceArgs& a, int i, int j, int periodic) {
    // x_j - x_i from the FP64 positions, minimum image when the force is periodic.
    float3 d = make_float3((float)(a.x[j] - a.x[i]), (float)(a.y[j] - a.y[i]),
                           (float)(a.z[j] - a.z[i]));
    if (periodic) {
        d.x -= a.box.x * rintf(d.x * a.inv_box.x);
        d.y -= a.box.y * rintf(d.y * a.inv_box.y);
        d.z -= a.box.z * rintf(d.z * a.inv_box.z);
    }
    return d;
}

template <int TERMS, bool PERIODIC, bool ENERGY>
__global__ void __launch_bounds__(kForceThreads) k_forces(ForceArgs a) {
    const int lane = threadIdx.x & 31;
    int blk = blockIdx.x;
    if (blk < a.blocks_tiles) {
        // ---------------- cluster-pair tiles ----------------
        // Warps take chunks of kTilesPerChunk consecutive tiles of the
        // flattened (row-major) tile list in a grid-stride loop, so every
        // SM holds many warps whatever the row lengths; the i-side force of
        // a row is flushed when the chunk crosses into the next row.
        // Fixed-point accumulation keeps the result independent of the split.
        const int total = a.tile_start[a.nc];
        if (total > a.tile_cap) return;  // overflowed list (flagged for a retry)
        const int gw = blk * kWarpsPerForceBlock + (threadIdx.x >> 5);
        const int stride = a.blocks_tiles * kWarpsPerForceBlock * kTilesPerChunk;
        const bool labels = a.pc.uses_labels != 0;
        double eacc[4] = {0.0, 0.0, 0.0, 0.0};
        for (int c0 = gw * kTilesPerChunk; c0 < total; c0 += stride) {
            const int c1 = min(total, c0 + kTilesPerChunk);
            int I = a.tile_i[c0];  // row of the chunk's first tile
            int row_end = a.tile_start[I + 1];
            int ki = I * 32 + lane;
            float4 xi = a.xs[ki];
            float4 p0i = a.p0s[ki];
            float4 p1i = (TERMS & kTermLJA) ? a.p1s[ki] : make_float4(0.f, 0.f, 0.f, 0.f);
            uint32_t labi = a.labs[ki];
            float3 fi = make_float3(0.f, 0.f, 0.f);
            for (int t = c0; t < c1; ++t) {
                while (t >= row_end) {
                    const int oi = a.perm[ki];
                    if (oi >= 0) add_force(a, oi, fi);
                    fi = make_float3(0.f, 0.f, 0.f);
                    ++I;
                    row_end = a.tile_start[I + 1];
                    ki = I * 32 + lane;
                    xi = a.xs[ki];
                    p0i = a.p0s[ki];
                    if (TERMS & kTermLJA) p1i = a.p1s[ki];
                    labi = a.labs[ki];
                }
                const int J = a.tile_j[t];
                const int m = a.tile_mask[t];
                const int kj = J * 32 + lane;
                float4 xj = a.xs[kj];
                const float4 sh = a.tile_shift[t];  // anchor shift, w: minimum image needed
                const float3 A = make_float3(sh.x, sh.y, sh.z);
                const bool wrap = PERIODIC && sh.w != 0.f;
                float4 p0j = a.p0s[kj];
                float4 p1j = (TERMS & kTermLJA) ? a.p1s[kj] : make_float4(0.f, 0.f, 0.f, 0.f);
                uint32_t labj = a.labs[kj];
                float3 fj = make_float3(0.f, 0.f, 0.f);
                uint32_t mw[4] = {0u, 0u, 0u, 0u};
                if (m >= 0) {
    #pragma unroll
                    for (int term = 0; term < 4; ++term)
                        if (TERMS & (1 << term)) mw[term] = a.masks[(size_t)m * 128 + term * 32 + lane];
                }
                const bool diag = (J == I);
                PairEnergy e;
                e.zero();
                for (int r = 0; r < 32; ++r) {
                    const bool do_pair = !diag || (r > 0 && (r < 16 || (r == 16 && lane < 16)));
                    if (do_pair) {
                        float3 d = anchored_sep(xi, xj, A);
                        if (wrap) d = min_image(d, a.box, a.inv_box);
                        const float r2 = norm2(d);
                        if (r2 < a.pc.list_rc2) {
                            uint32_t ex = a.excl_all;
                            if (m >= 0) {  // the tile holds excluded pairs
    #pragma unroll
                                for (int term = 0; term < 4; ++term)
                                    if (TERMS & (1 << term)) ex |= ((mw[term] >> r) & 1u) << term;
                            }
                            if (labels) {
    #pragma unroll
                                for (int term = 0; term < 4; ++term)
                                    if ((TERMS & (1 << term)) && (a.pc.uses_labels & (1 << term)) &&
                                        !labels_allow(labi, labj, term, a.pc.allow[term]))
                                        ex |= 1u << term;
                            }
                            const float s = pair_scalar<TERMS, ENERGY>(r2, p0i, p0j, p1i, p1j, ex, a.pc, e);
                            fi.x -= s * d.x;
                            fi.y -= s * d.y;
                            fi.z -= s * d.z;
                            fj.x += s * d.x;
                            fj.y += s * d.y;
                            fj.z += s * d.z;
                        }
                    }
                    const int src = (lane + 1) & 31;
                    xj = shfl4(xj, src);
                    if (TERMS & kTermEXV) p0j.x = __shfl_sync(kFull, p0j.x, src);
                    if (TERMS & kTermDH) p0j.y = __shfl_sync(kFull, p0j.y, src);
                    if (TERMS & kTermLJR) {
                        p0j.z = __shfl_sync(kFull, p0j.z, src);
                        p0j.w = __shfl_sync(kFull, p0j.w, src);
                    }
                    if (TERMS & kTermLJA) {
                        p1j.x = __shfl_sync(kFull, p1j.x, src);
                        if (!(TERMS & kLJSameSigma)) p1j.y = __shfl_sync(kFull, p1j.y, src);
                    }
                    if (labels) labj = __shfl_sync(kFull, labj, src);
                    fj.x = __shfl_sync(kFull, fj.x, src);
                    fj.y = __shfl_sync(kFull, fj.y, src);
                    fj.z = __shfl_sync(kFull, fj.z, src);
                }
                const int oj = a.perm[kj];
                if (oj >= 0) add_force(a, oj, fj);
                if (ENERGY) {
                    eacc[0] += e.exv;
                    eacc[1] += e.dh;
                    eacc[2] += e.ljr;
                    eacc[3] += e.lja;
                }
            }
            const int oi = a.perm[ki];
            if (oi >= 0) add_force(a, oi, fi);
        }
        if (ENERGY) {
#pragma unroll
            for (int term = 0; term < 4; ++term) {
                if (!(TERMS & (1 << term))) continue;
                const double v = warp_sum(eacc[term]);
                if (lane == 0 && v != 0.0) atomicAdd(&a.energy[term], v);
            }
        }
        return;
    }
    blk -= a.blocks_tiles;
    if (blk < a.blocks_bonds) {
        // ------------ harmonic bonds, Go contacts, Gaussian bonds ------------
        const int t = blk * kForceThreads + threadIdx.x;
        float eh = 0.f, eg = 0.f, eb = 0.f, ec = 0.f;
        if (t < a.n_bonds) {
            const BondTerm b = a.bonds[t];
            const int slot = bond_slot(b.kind);
            if (a.slots_enabled & (1u << slot)) {
                double dx = a.x[b.j] - a.x[b.i], dy = a.y[b.j] - a.y[b.i], dz = a.z[b.j] - a.z[b.i];
                if (b.periodic) {
                    dx -= (double)a.box.x * rint(dx * (double)a.inv_box.x);
                    dy -= (double)a.box.y * rint(dy * (double)a.inv_box.y);
                    dz -= (double)a.box.z * rint(dz * (double)a.inv_box.z);
                }
                const double r2d = dx * dx + dy * dy + dz * dz;
                const float delta = (float)(r2d - ((double)b.r0sq_hi + (double)b.r0sq_lo));
                const float3 d = make_float3((float)dx, (float)dy, (float)dz);
                float en;
                const float s = bond_scalar(b.kind, norm2(d), delta, b.p0, b.p1, b.r0sq_hi, en);
                add_force(a, b.i, make_float3(-s * d.x, -s * d.y, -s * d.z));
                add_force(a, b.j, make_float3(s * d.x, s * d.y, s * d.z));
                if (b.kind == kBondHarmonic) eh = en;
                else if (b.kind == kBondGo) eg = en;
                else if (b.kind == kBondGauss) eb = en;
                else ec = en;
            }
        }
        if (ENERGY) {
            const double vh = warp_sum((double)eh), vg = warp_sum((double)eg), vb = warp_sum((double)eb),
                         vc = warp_sum((double)ec);
            if (lane == 0) {
                if (vh != 0.0) atomicAdd(&a.energy[kSlotHB], vh);
                if (vg != 0.0) atomicAdd(&a.energy[kSlotGO], vg);
                if (vb != 0.0) atomicAdd(&a.energy[kSlotGB], vb);
                if (vc != 0.0) atomicAdd(&a.energy[kSlotCGO], vc);
            }
        }
        return;
    }
    blk -= a.blocks_bonds;
    if (blk < a.blocks_angles) {
        const int t = blk * kForceThreads + threadIdx.x;
        float en = 0.f;
        if (t < a.n_angles && (a.slots_enabled & (1u << kSlotFLA))) {
            const AngleTerm g = a.angles[t];
            const float3 u = bonded_sep(a, g.j, g.i, g.periodic);  // x1 - x2
            const float3 v = bonded_sep(a, g.j, g.k, g.periodic);  // x3 - x2
            float3 f1, f3;
            fla_forces(u, v, g.kk, a.fla[g.table], f1, f3, en);
            add_force(a, g.i, f1);
            add_force(a, g.k, f3);
            add_force(a, g.j, make_float3(-f1.x - f3.x, -f1.y - f3.y, -f1.z - f3.z));
        }
        if (ENERGY) {
            const double v = warp_sum((double)en);
            if (lane == 0 && v != 0.0) atomicAdd(&a.energy[kSlotFLA], v);
        }
        return;
    }
    blk -= a.blocks_angles;
    if (blk < a.blocks_dih) {
        const int t = blk * kForceThreads + threadIdx.x;
        float efld = 0.f, egd = 0.f;
        if (t < a.n_dih) {
            const DihedralTerm q = a.dih[t];
            const int slot = q.kind == kDihFLD ? kSlotFLD : kSlotGD;
            if (a.slots_enabled & (1u << slot)) {
                const float3 F = bonded_sep(a, q.j, q.i, q.periodic);  // x1 - x2
                const float3 G = bonded_sep(a, q.k, q.j, q.periodic);  // x2 - x3
                const float3 H = bonded_sep(a, q.k, q.l, q.periodic);  // x4 - x3
                float3 f1, f2, f3, f4;
                float en;
                if (q.kind == kDihFLD) {
                    fld_forces(F, G, H, q.kk, a.fld[q.table], f1, f2, f3, f4, en);
                    efld = en;
                } else {
                    gauss_dihedral_forces(F, G, H, q.kk, q.theta0, q.inv2s2, f1, f2, f3, f4, en);
                    egd = en;
                }
                add_force(a, q.i, f1);
                add_force(a, q.j, f2);
                add_force(a, q.k, f3);
                add_force(a, q.l, f4);
            }
        }
        if (ENERGY) {
            const double v = warp_sum((double)efld), vg = warp_sum((double)egd);
            if (lane == 0) {
                if (v != 0.0) atomicAdd(&a.energy[kSlotFLD], v);
                if (vg != 0.0) atomicAdd(&a.energy[kSlotGD], vg);
            }
        }
        return;
    }
    blk -= a.blocks_dih;
    {
        // ---------------- charged pairs (Debye-Hueckel) ----------------
        // One warp per charged bead over its row; each pair's force on bead
        // i is rounded to fixed point and summed as integers, then added
        // once per bead.
        const int warp = threadIdx.x >> 5;
        float edh = 0.f;
        if (a.slots_enabled & (1u << kSlotDH)) {
            const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
            for (int t = blk * kWarpsPerForceBlock + warp; t < a.n_chg; t += a.blocks_chg * kWarpsPerForceBlock) {
                const int i = a.chg_idx[t];
                const float4 xi = a.xq[i], li = a.xlo[i];
                const float4 pi = a.p0[i];
                const int len = min(a.chg_len[t], a.chg_row_cap);
                const int32_t* row = a.chg_rows + (size_t)t * a.chg_row_cap;
                long long fx = 0, fy = 0, fz = 0;
                bool bad = false;
                for (int p = lane; p < len; p += 32) {
                    const int j = row[p];
                    const float3 d = ff_separation<PERIODIC>(xi, li, a.xq[j], a.xlo[j], a.box, a.inv_box);
                    const float r2 = norm2(d);
                    if (r2 < a.pc.dh_rc2) {
                        PairEnergy e;
                        e.zero();
                        const float sc = pair_scalar<kTermDH, ENERGY>(r2, pi, a.p0[j], zero4, zero4, 0u, a.pc, e);
                        bad = bad || !force_ok(make_float3(sc * d.x, sc * d.y, sc * d.z));
                        fx += (long long)to_fixed(-sc * d.x);
                        fy += (long long)to_fixed(-sc * d.y);
                        fz += (long long)to_fixed(-sc * d.z);
                        if (ENERGY && i < j) edh += e.dh;
                    }
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    fx += __shfl_xor_sync(0xffffffffu, fx, o);
                    fy += __shfl_xor_sync(0xffffffffu, fy, o);
                    fz += __shfl_xor_sync(0xffffffffu, fz, o);
                }
                if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(a.flags, ListFlags::kBlownUp);
                if (lane == 0) {
                    if (fx) atomicAdd(&a.F[i], (unsigned long long)fx);
                    if (fy) atomicAdd(&a.F[a.n + i], (unsigned long long)fy);
                    if (fz) atomicAdd(&a.F[2 * a.n + i], (unsigned long long)fz);
                }
            }
        }
        if (ENERGY) {
            const double v = warp_sum((double)edh);
            if (lane == 0 && v != 0.0) atomicAdd(&a.energy[kSlotDH], v);
        }
    }
}

// ---------------------------------------------------------------------------
// Langevin integrator (OpenMM LangevinIntegrator, leapfrog form):
//   v <- vscale v + fscale F/m + noise sqrt(1/m) N(0,1);  x <- x + v dt
// ---------------------------------------------------------------------------
struct IntegrateArgs {
    int n;
    unsigned long long* F;
    float *vx, *vy, *vz;
    double *x, *y, *z;
    const float* invm;
    float4 *xq, *xlo, *xs;
    const float4* anc;
    const int32_t* slot;
    const float4* ref;
    LangevinConsts lc;
    const unsigned long long* step_base;
    int r;
    int periodic;
    double box[3], inv_box[3];
    float3 fbox, finv_box;
    float disp_limit2;
    int32_t* flags;
};


__global__ void k_integrate(IntegrateArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const unsigned long long step = *a.step_base + (unsigned long long)a.r;
    const float fx = fixed_to_float((long long)a.F[i]);
    const float fy = fixed_to_float((long long)a.F[a.n + i]);
    const float fz = fixed_to_float((long long)a.F[2 * a.n + i]);
    bool bad = !(fabsf(fx) < kForceLimit && fabsf(fy) < kForceLimit && fabsf(fz) < kForceLimit);
    a.F[i] = 0ull;
    a.F[a.n + i] = 0ull;
    a.F[2 * a.n + i] = 0ull;
    const float im = a.invm[i];
    double x = a.x[i], y = a.y[i], z = a.z[i];
    if (im > 0.f) {
        const float3 g = gaussian3(a.lc.seed, a.lc.stream, (uint32_t)i, step, kPurposeLangevin);
        const float sq = sqrtf(im) * a.lc.noise;
        const float fs = a.lc.fscale * im;
        const float vx = a.lc.vscale * a.vx[i] + fs * fx + sq * g.x;
        const float vy = a.lc.vscale * a.vy[i] + fs * fy + sq * g.y;
        const float vz = a.lc.vscale * a.vz[i] + fs * fz + sq * g.z;
        a.vx[i] = vx;
        a.vy[i] = vy;
        a.vz[i] = vz;
        x += (double)vx * (double)a.lc.dt;
        y += (double)vy * (double)a.lc.dt;
        z += (double)vz * (double)a.lc.dt;
        a.x[i] = x;
        a.y[i] = y;
        a.z[i] = z;
        bad = bad || !(isfinite(x) && isfinite(y) && isfinite(z));
    }
    if (bad) atomicOr(a.flags, ListFlags::kBlownUp);
    double w[3] = {x, y, z};
    if (a.periodic)
        for (int c = 0; c < 3; ++c) w[c] = wrap_coord(w[c], a.box[c], a.inv_box[c]);
    const float4 p = make_float4(__double2float_rn(w[0]), __double2float_rn(w[1]), __double2float_rn(w[2]), 0.f);
    a.xq[i] = p;
    a.xlo[i] = make_float4(__double2float_rn(__dsub_rn(w[0], (double)p.x)),
                           __double2float_rn(__dsub_rn(w[1], (double)p.y)),
                           __double2float_rn(__dsub_rn(w[2], (double)p.z)), 0.f);
    const int k = a.slot[i];
    const float4 an = a.anc[k >> 5];
    a.xs[k] = make_float4(anchor_offset(w[0], an.x, a.box[0], a.inv_box[0], a.periodic),
                          anchor_offset(w[1], an.y, a.box[1], a.inv_box[1], a.periodic),
                          anchor_offset(w[2], an.z, a.box[2], a.inv_box[2], a.periodic), 0.f);
    const float4 q = a.ref[i];
    float3 d = a.periodic ? separation<true>(q, p, a.fbox, a.finv_box)
                          : separation<false>(q, p, a.fbox, a.finv_box);
    const float d2 = norm2(d);
    if (d2 > a.disp_limit2) atomicOr(a.flags, ListFlags::kSkinViolation);
}

__global__ void k_positions_to_float(int n, const double* __restrict__ x,
                                     const double* __restrict__ y, const double* __restrict__ z,
                                     int periodic, double bx, double by, double bz, double ibx,
                                     double iby, double ibz, float4* __restrict__ xq,
                                     float4* __restrict__ xlo) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double w[3] = {x[i], y[i], z[i]};
    if (periodic) {
        w[0] = wrap_coord(w[0], bx, ibx);
        w[1] = wrap_coord(w[1], by, iby);
        w[2] = wrap_coord(w[2], bz, ibz);
    }
    const float4 p = make_float4(__double2float_rn(w[0]), __double2float_rn(w[1]), __double2float_rn(w[2]), 0.f);
    xq[i] = p;
    xlo[i] = make_float4(__double2float_rn(__dsub_rn(w[0], (double)p.x)),
                         __double2float_rn(__dsub_rn(w[1], (double)p.y)),
                         __double2float_rn(__dsub_rn(w[2], (double)p.z)), 0.f);
}

__global__ void k_advance(unsigned long long* step_base, unsigned long long k) { *step_base += k; }

__global__ void k_velocity_init(int n, const float* __restrict__ invm, float kT, uint32_t seed,
                                uint32_t stream, float* vx, float* vy, float* vz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float im = invm[i];
    const float3 g = gaussian3(seed, stream, (uint32_t)i, 0ull, kPurposeVelocityInit);
    const float s = im > 0.f ? sqrtf(kT * im) : 0.f;
    vx[i] = s * g.x;
    vy[i] = s * g.y;
    vz[i] = s * g.z;
}

__global__ void k_kinetic(int n, const float* __restrict__ invm, const float* __restrict__ vx,
                          const float* __restrict__ vy, const float* __restrict__ vz, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0.0;
    if (i < n && invm[i] > 0.f) {
        const double m = 1.0 / (double)invm[i];
        e = 0.5 * m * ((double)vx[i] * vx[i] + (double)vy[i] * vy[i] + (double)vz[i] * vz[i]);
    }
    e = warp_sum(e);
    if ((threadIdx.x & 31) == 0 && e != 0.0) atomicAdd(out, e);
}

// Verification: emit every pair the tiles make the kernel test whose FP32
// r^2 is below the largest cutoff squared.
template <bool PERIODIC>
__global__ void k_list_pairs(int nc, const float4* __restrict__ xs, const float4* __restrict__ tile_shift,
                             const int32_t* __restrict__ perm,
                             const int32_t* __restrict__ tile_start, const int32_t* __restrict__ tile_j,
                             float3 box, float3 inv_box, float rc2, long long* out, long long cap,
                             unsigned long long* count, long long tile_cap) {
    const int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (I >= nc) return;
    if ((long long)tile_start[nc] > tile_cap) return;
    const float4 xi = xs[I * 32 + lane];
    const int oi = perm[I * 32 + lane];
    for (int t = tile_start[I]; t < tile_start[I + 1]; ++t) {
        const int J = tile_j[t];
        const bool diag = J == I;
        const float3 A = make_float3(tile_shift[t].x, tile_shift[t].y, tile_shift[t].z);
        for (int r = 0; r < 32; ++r) {
            const int jl = (lane + r) & 31;
            const bool do_pair = !diag || (r > 0 && (r < 16 || (r == 16 && lane < 16)));
            const float4 xj = xs[J * 32 + jl];
            const int oj = perm[J * 32 + jl];
            if (do_pair && oi >= 0 && oj >= 0) {
                float3 d = anchored_sep(xi, xj, A);
                if (PERIODIC) d = min_image(d, box, inv_box);
                const float r2 = norm2(d);
                if (r2 < rc2) {
                    const unsigned long long at = atomicAdd(count, 1ull);
                    if ((long long)at < cap) {
                        out[2 * at] = min(oi, oj);
                        out[2 * at + 1] = max(oi, oj);
                    }
                }
            }
        }
    }
}

template <int TERMS>
void launch_forces_t(const ForceArgs& a, int grid, cudaStream_t s, bool periodic, bool energy) {
    if (periodic) {
        if (energy) k_forces<TERMS, true, true><<<grid, kForceThreads, 0, s>>>(a);
        else k_forces<TERMS, true, false><<<grid, kForceThreads, 0, s>>>(a);
    } else {
        if (energy) k_forces<TERMS, false, true><<<grid, kForceThreads, 0, s>>>(a);
        else k_forces<TERMS, false, false><<<grid, kForceThreads, 0, s>>>(a);
    }
}

inline int div_up(int64_t a, int b) { return (int)((a + b - 1) / b); }

}  // namespace

// ===========================================================================
// PlainContext
// ===========================================================================
PlainContext::PlainContext(const SystemDesc& d, double temperature, double friction, double dt,
                           int32_t seed, int dev)
    : device(dev) {
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
        throw Error(2, "[error] no CUDA device is available");
    if (dev < 0 || dev >= count) throw Error(1, "[error] invalid device index");
    OCM_CK(cudaSetDevice(dev));
    OCM_CK(cudaDeviceGetAttribute(&num_sms_, cudaDevAttrMultiProcessorCount, dev));
    if (!(dt > 0)) throw Error(1, "[error] step size must be positive");
    if (!(friction >= 0)) throw Error(1, "[error] friction must be >= 0");
    if (!(temperature >= 0)) throw Error(1, "[error] temperature must be >= 0");
    cs = compile_system(d);
    desc_ = d;
    one_seed_ = seed;
    one_T_ = temperature;
    one_friction_ = friction;
    one_dt_ = dt;
    n = cs.n;
    if (n <= 0) throw Error(1, "[error] system has no particles");
    if (n > (1 << 27)) throw Error(6, "[error] system too large");
    OCM_CK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    OCM_CK(cudaMallocHost(&h_flags_, 16 * sizeof(int32_t)));

    // Langevin constants (OpenMM LangevinIntegrator).
    const double vscale = std::exp(-friction * dt);
    const double fscale = friction == 0 ? dt : (1.0 - vscale) / friction;
    const double kT = constant::boltz * temperature;
    lc_.vscale = (float)vscale;
    lc_.fscale = (float)fscale;
    lc_.noise = (float)std::sqrt(kT * (1.0 - vscale * vscale));
    lc_.dt = (float)dt;
    lc_.seed = (uint32_t)seed;
    lc_.stream = 0u;

    box_ = make_float3((float)cs.box[0], (float)cs.box[1], (float)cs.box[2]);
    inv_box_ = make_float3(cs.box[0] > 0 ? (float)(1.0 / cs.box[0]) : 0.f,
                           cs.box[1] > 0 ? (float)(1.0 / cs.box[1]) : 0.f,
                           cs.box[2] > 0 ? (float)(1.0 / cs.box[2]) : 0.f);
    reorder = cs.periodic && n > 2048;
    np = ((n + 31) / 32) * 32;
    if (reorder) {
        // Columns at least this wide number at most n / 32, so the padding of
        // each column to whole clusters at most doubles the slots.
        col_wmin_ = std::max(1.0, std::sqrt(cs.box[0] * cs.box[1] * 32.0 / (double)n));
        const int64_t max_cols = (int64_t)std::max(1.0, std::floor(cs.box[0] / col_wmin_)) *
                                 (int64_t)std::max(1.0, std::floor(cs.box[1] / col_wmin_));
        np += 32 * max_cols;
    }
    nc = np / 32;

    cudaStream_t s = stream_;
    x_.alloc(n); y_.alloc(n); z_.alloc(n);
    vx_.alloc(n); vy_.alloc(n); vz_.alloc(n);
    OCM_CK(cudaMemsetAsync(vx_.p, 0, n * sizeof(float), s));
    OCM_CK(cudaMemsetAsync(vy_.p, 0, n * sizeof(float), s));
    OCM_CK(cudaMemsetAsync(vz_.p, 0, n * sizeof(float), s));
    invm_.upload(cs.inv_mass, s);
    F_.alloc(3 * n);
    OCM_CK(cudaMemsetAsync(F_.p, 0, 3 * n * sizeof(unsigned long long), s));
    xq_.alloc(n); xlo_.alloc(n); ref_.alloc(n);
    {
        std::vector<float4> p0(n), p1(n);
        for (int64_t i = 0; i < n; ++i) {
            p0[i] = make_float4(cs.p0[4 * i], cs.p0[4 * i + 1], cs.p0[4 * i + 2], cs.p0[4 * i + 3]);
            p1[i] = make_float4(cs.p1[4 * i], cs.p1[4 * i + 1], cs.p1[4 * i + 2], cs.p1[4 * i + 3]);
        }
        p0_.upload(p0, s);
        p1_.upload(p1, s);
    }
    lab_.upload(cs.labels, s);
    slot_.alloc(n);
    perm_.alloc(np);
    {
        std::vector<int32_t> id(np);
        for (int64_t k = 0; k < np; ++k) id[k] = k < n ? (int32_t)k : -1;
        perm_.upload(id, s);
    }
    xs_.alloc(np); p0s_.alloc(np); p1s_.alloc(np); labs_.alloc(np);
    bb_c_.alloc(nc); bb_h_.alloc(nc); anc_.alloc(nc); ext_.alloc(nc);
    tile_count_.alloc(nc); tile_start_.alloc(nc + 1); raw_start_.alloc(nc + 1);
    tile_cap_ = std::min<int64_t>(nc * (nc + 1) / 2, std::max<int64_t>(4096, nc * 48));
    alloc_tile_arrays();
    mask_cap_ = std::max<int64_t>(256, std::min<int64_t>(tile_cap_, nc * 8));
    masks_.alloc(mask_cap_ * 128);
    mask_count_.alloc(1);

    if (reorder) {
        cell_key_.alloc(n);
        bucket_.alloc(n);
        setup_columns(std::max(col_wmin_, 2.5));  // until positions give the density
    }
    // exclusions (CSR -> flat (i, j, bits))
    {
        std::vector<int32_t> ei(cs.ex_j.size());
        for (int64_t i = 0; i < n; ++i)
            for (int32_t e = cs.ex_start[i]; e < cs.ex_start[i + 1]; ++e) ei[e] = (int32_t)i;
        ex_start_.upload(ei, s);  // row index of each entry
        ex_j_.upload(cs.ex_j, s);
        ex_bits_.upload(cs.ex_bits, s);
        ex_csr_.upload(cs.ex_start, s);
    }
    // Charged-pair list: worth it when the Debye-Hueckel cutoff clearly
    // exceeds the other pair cutoffs (most of the tiles' volume would serve
    // the few charged pairs only) and no interaction groups restrict it.
    tile_cutoff_ = cs.max_cutoff;
    {
        const PairConsts& pc = cs.pc;
        double other = 0.0;
        if (pc.terms & kTermEXV) other = std::max(other, std::sqrt((double)pc.exv_rc2));
        if (pc.terms & kTermLJR) other = std::max(other, std::sqrt((double)pc.ljr_rc2));
        if (pc.terms & kTermLJA) other = std::max(other, std::sqrt((double)pc.lja_rc2));
        const double dh = (pc.terms & kTermDH) ? std::sqrt((double)pc.dh_rc2) : 0.0;
        std::vector<int32_t> idx;
        for (int64_t i = 0; i < n; ++i)
            if (cs.p0[4 * i + 1] != 0.f) idx.push_back((int32_t)i);
        if (reorder && cs.periodic && (pc.terms & kTermDH) && !(pc.uses_labels & kTermDH) && dh > other + 0.3 &&
            !idx.empty()) {
            n_charged_ = (int64_t)idx.size();
            chg_idx_.upload(idx, s);
            chg_key_.alloc(n_charged_);
            chg_sorted_.alloc(n_charged_);
            chg_len_.alloc(n_charged_);
            OCM_CK(cudaMemsetAsync(chg_len_.p, 0, n_charged_ * sizeof(int32_t), s));
            chg_stats_.alloc(2);
            OCM_CK(cudaMemsetAsync(chg_stats_.p, 0, 2 * sizeof(int32_t), s));
            charged_split_ = true;
            tile_cutoff_ = other;
            setup_charged_cells();
            if (charged_split_) {
                chg_row_cap_ = 128;
                chg_rows_.alloc(n_charged_ * chg_row_cap_);
            }
        }
    }
    bonds_.upload(cs.bonds, s);
    angles_.upload(cs.angles, s);
    dihedrals_.upload(cs.dihedrals, s);
    fla_.upload(cs.fla, s);
    fld_.upload(cs.fld, s);
    energy_.alloc(kNumSlots);
    flags_.alloc(1);
    OCM_CK(cudaMemsetAsync(flags_.p, 0, sizeof(int32_t), s));
    step_base_.alloc(1);
    OCM_CK(cudaMemsetAsync(step_base_.p, 0, sizeof(unsigned long long), s));
    ke_.alloc(1);
    sx_.alloc(n); sy_.alloc(n); sz_.alloc(n);
    svx_.alloc(n); svy_.alloc(n); svz_.alloc(n);
    sstep_.alloc(1);
    OCM_CK(cudaStreamSynchronize(s));
}

PlainContext::~PlainContext() {
    cudaSetDevice(device);
    clear_graphs();
    if (stream_) cudaStreamSynchronize(stream_);
    if (h_flags_) cudaFreeHost(h_flags_);
    if (stream_) cudaStreamDestroy(stream_);
}

void PlainContext::clear_graphs() {
    for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
    graphs_.clear();
}

void PlainContext::check_positions_set() const {
    if (!positions_set_) throw Error(5, "[error] positions have not been set");
}

void PlainContext::set_positions(const double* xyz) { set_positions_impl(xyz, true); }
void PlainContext::set_positions_internal(const double* xyz) { set_positions_impl(xyz, false); }

void PlainContext::set_positions_impl(const double* xyz, bool retune) {
    OCM_CK(cudaSetDevice(device));
    std::vector<double> a(n), b(n), c(n);
    for (int64_t i = 0; i < n; ++i) {
        a[i] = xyz[3 * i];
        b[i] = xyz[3 * i + 1];
        c[i] = xyz[3 * i + 2];
        if (!std::isfinite(a[i]) || !std::isfinite(b[i]) || !std::isfinite(c[i]))
            throw Error(7, "[error] non-finite position for particle " + std::to_string(i));
    }
    if (reorder && retune) {
        // Bead density over the occupied 1 nm cells sets the column width:
        // clusters of 32 beads then come out about as tall as wide.
        int g[3];
        for (int k = 0; k < 3; ++k) g[k] = (int)std::max(1.0, std::min(1024.0, std::floor(cs.box[k])));
        std::vector<int64_t> cells(n);
        const double* v[3] = {a.data(), b.data(), c.data()};
        for (int64_t i = 0; i < n; ++i) {
            int64_t key = 0;
            for (int k = 0; k < 3; ++k) {
                const double w = v[k][i] - cs.box[k] * std::floor(v[k][i] / cs.box[k]);
                key = key * 1024 + std::min<int64_t>(g[k] - 1, std::max<int64_t>(0, (int64_t)(w * g[k] / cs.box[k])));
            }
            cells[i] = key;
        }
        std::sort(cells.begin(), cells.end());
        const int64_t occupied = std::unique(cells.begin(), cells.end()) - cells.begin();
        const double cell_vol = cs.box[0] * cs.box[1] * cs.box[2] / ((double)g[0] * g[1] * g[2]);
        const double density = (double)n / ((double)occupied * cell_vol);
        setup_columns(1.2 * std::cbrt(32.0 / density));
    }
    x_.upload(a, stream_);
    y_.upload(b, stream_);
    z_.upload(c, stream_);
    k_positions_to_float<<<div_up(n, 256), 256, 0, stream_>>>(
        (int)n, x_.p, y_.p, z_.p, cs.periodic ? 1 : 0, cs.box[0], cs.box[1], cs.box[2],
        cs.box[0] > 0 ? 1.0 / cs.box[0] : 0.0, cs.box[1] > 0 ? 1.0 / cs.box[1] : 0.0,
        cs.box[2] > 0 ? 1.0 / cs.box[2] : 0.0, xq_.p, xlo_.p);
    OCM_CK(cudaGetLastError());
    OCM_CK(cudaStreamSynchronize(stream_));
    positions_set_ = true;
}

void PlainContext::get_positions(double* xyz) {
    OCM_CK(cudaSetDevice(device));
    check_positions_set();
    std::vector<double> a(n), b(n), c(n);
    OCM_CK(cudaMemcpyAsync(a.data(), x_.p, n * sizeof(double), cudaMemcpyDeviceToHost, stream_));
    OCM_CK(cudaMemcpyAsync(b.data(), y_.p, n * sizeof(double), cudaMemcpyDeviceToHost, stream_));
    OCM_CK(cudaMemcpyAsync(c.data(), z_.p, n * sizeof(double), cudaMemcpyDeviceToHost, stream_));
    OCM_CK(cudaStreamSynchronize(stream_));
    for (int64_t i = 0; i < n; ++i) {
        xyz[3 * i] = a[i];
        xyz[3 * i + 1] = b[i];
        xyz[3 * i + 2] = c[i];
    }
}

void PlainContext::set_velocities(const double* v) {
    OCM_CK(cudaSetDevice(device));
    std::vector<float> a(n), b(n), c(n);
    for (int64_t i = 0; i < n; ++i) {
        a[i] = (float)v[3 * i];
        b[i] = (float)v[3 * i + 1];
        c[i] = (float)v[3 * i + 2];
    }
    vx_.upload(a, stream_);
    vy_.upload(b, stream_);
    vz_.upload(c, stream_);
    OCM_CK(cudaStreamSynchronize(stream_));
}

void PlainContext::get_velocities(double* v) {
    OCM_CK(cudaSetDevice(device));
    std::vector<float> a(n), b(n), c(n);
    OCM_CK(cudaMemcpyAsync(a.data(), vx_.p, n * sizeof(float), cudaMemcpyDeviceToHost, stream_));
    OCM_CK(cudaMemcpyAsync(b.data(), vy_.p, n * sizeof(float), cudaMemcpyDeviceToHost, stream_));
    OCM_CK(cudaMemcpyAsync(c.data(), vz_.p, n * sizeof(float), cudaMemcpyDeviceToHost, stream_));
    OCM_CK(cudaStreamSynchronize(stream_));
    for (int64_t i = 0; i < n; ++i) {
        v[3 * i] = a[i];
        v[3 * i + 1] = b[i];
        v[3 * i + 2] = c[i];
    }
}

void PlainContext::set_velocities_to_temperature(double temperature, int32_t seed) {
    OCM_CK(cudaSetDevice(device));
    const float kT = (float)(constant::boltz * temperature);
    k_velocity_init<<<div_up(n, 256), 256, 0, stream_>>>((int)n, invm_.p, kT, (uint32_t)seed, 1u,
                                                         vx_.p, vy_.p, vz_.p);
    OCM_CK(cudaGetLastError());
    OCM_CK(cudaStreamSynchronize(stream_));
}

double PlainContext::kinetic_energy() {
    OCM_CK(cudaSetDevice(device));
    OCM_CK(cudaMemsetAsync(ke_.p, 0, sizeof(double), stream_));
    k_kinetic<<<div_up(n, 256), 256, 0, stream_>>>((int)n, invm_.p, vx_.p, vy_.p, vz_.p, ke_.p);
    OCM_CK(cudaGetLastError());
    double ke = 0;
    OCM_CK(cudaMemcpyAsync(&ke, ke_.p, sizeof(double), cudaMemcpyDeviceToHost, stream_));
    OCM_CK(cudaStreamSynchronize(stream_));
    return ke;
}

void PlainContext::rebuild(cudaStream_t s) {
    const int np_i = (int)np, n_i = (int)n, nc_i = (int)nc;
    if (reorder) {
        const int ncols = cell_dims_[0] * cell_dims_[1];
        // the charged beads' cell sort rides along in the same launches
        const int m = charged_split_ ? (int)n_charged_ : 0;
        OCM_CK(cudaMemsetAsync(cell_count_.p, 0, n_cells_ * sizeof(int32_t), s));
        OCM_CK(cudaMemsetAsync(cell_fill_.p, 0, n_cells_ * sizeof(int32_t), s));
        OCM_CK(cudaMemsetAsync(perm_.p, 0xff, np * sizeof(int32_t), s));
        if (m > 0) {
            OCM_CK(cudaMemsetAsync(chg_count_.p, 0, n_charged_cells_ * sizeof(int32_t), s));
            OCM_CK(cudaMemsetAsync(chg_fill_.p, 0, n_charged_cells_ * sizeof(int32_t), s));
            OCM_CK(cudaMemsetAsync(chg_stats_.p, 0, 2 * sizeof(int32_t), s));
        }
        k_keys_both<<<div_up(n + m, 256), 256, 0, s>>>(n_i, xq_.p, cell_dims_[0], cell_dims_[1], cell_dims_[2],
                                                       box_, cell_key_.p, cell_count_.p, m, chg_idx_.p,
                                                       charged_cells_[0], charged_cells_[1], charged_cells_[2],
                                                       chg_key_.p, chg_count_.p);
        if (m > 0)
            k_scan2<<<2, 1024, 0, s>>>((int)n_cells_, cell_count_.p, cell_start_.p, (int)n_charged_cells_,
                                       chg_count_.p, chg_start_.p);
        else
            k_scan<<<1, 1024, 0, s>>>((int)n_cells_, cell_count_.p, cell_start_.p);
        k_col_scan<<<1, 1024, 0, s>>>(ncols, cell_dims_[2], cell_start_.p, col_start_.p);
        k_scatter_both<<<div_up(n + m, 256), 256, 0, s>>>(n_i, cell_key_.p, cell_start_.p, cell_fill_.p,
                                                          bucket_.p, m, chg_idx_.p, chg_key_.p, xq_.p,
                                                          chg_start_.p, chg_fill_.p, chg_sorted_.p);
        k_bucket_rank<<<div_up(n, 256), 256, 0, s>>>(n_i, cell_dims_[2], cell_key_.p, cell_start_.p,
                                                     col_start_.p, bucket_.p, perm_.p);
    }
    const BoxD bd = box_d();
    k_gather_sorted<<<div_up(np, 256), 256, 0, s>>>(np_i, perm_.p, xq_.p, x_.p, y_.p, z_.p, bd, p0_.p, p1_.p,
                                                    lab_.p, slot_.p, xs_.p, anc_.p, p0s_.p, p1s_.p, labs_.p,
                                                    ref_.p);
    const bool per = cs.periodic;
    const int wblocks = div_up(nc * 32, 128);
    k_bbox<<<wblocks, 128, 0, s>>>(nc_i, xs_.p, anc_.p, perm_.p, bb_c_.p, bb_h_.p);
    k_reanchor<<<div_up(np, 128), 128, 0, s>>>(np_i, perm_.p, x_.p, y_.p, z_.p, bd, bb_c_.p, anc_.p, xs_.p,
                                               ext_.p);
    const float cut = (float)(tile_cutoff_ + skin) * 1.0001f + 1e-4f;
    const float cut2 = cut * cut;
    if (per) {
        k_tiles<true, false><<<wblocks, 128, 0, s>>>(nc_i, bb_c_.p, bb_h_.p, box_, inv_box_, cut, cut2,
                                                     tile_count_.p, nullptr, nullptr, nullptr, 0, flags_.p);
    } else {
        k_tiles<false, false><<<wblocks, 128, 0, s>>>(nc_i, bb_c_.p, bb_h_.p, box_, inv_box_, cut,
                                                      cut2, tile_count_.p, nullptr, nullptr, nullptr, 0, flags_.p);
    }
    k_scan<<<1, 1024, 0, s>>>(nc_i, tile_count_.p, raw_start_.p);
    OCM_CK(cudaMemsetAsync(tile_count_.p, 0, nc * sizeof(int32_t), s));
    const int pblocks = div_up(tile_cap_ * 32, 128);  // one warp per candidate tile
    if (per) {
        k_tiles<true, true><<<wblocks, 128, 0, s>>>(nc_i, bb_c_.p, bb_h_.p, box_, inv_box_, cut, cut2, nullptr,
                                                    raw_start_.p, raw_i_.p, raw_j_.p, (int)tile_cap_, flags_.p);
        k_prune<true><<<pblocks, 128, 0, s>>>(nc_i, xs_.p, anc_.p, raw_start_.p, raw_i_.p, raw_j_.p, (int)tile_cap_,
                                              box_, inv_box_, cut2, keep_.p, tile_count_.p);
    } else {
        k_tiles<false, true><<<wblocks, 128, 0, s>>>(nc_i, bb_c_.p, bb_h_.p, box_, inv_box_, cut, cut2,
                                                     nullptr, raw_start_.p, raw_i_.p, raw_j_.p, (int)tile_cap_,
                                                     flags_.p);
        k_prune<false><<<pblocks, 128, 0, s>>>(nc_i, xs_.p, anc_.p, raw_start_.p, raw_i_.p, raw_j_.p, (int)tile_cap_,
                                               box_, inv_box_, cut2, keep_.p, tile_count_.p);
    }
    k_scan<<<1, 1024, 0, s>>>(nc_i, tile_count_.p, tile_start_.p);
    k_compact_tiles<<<wblocks, 128, 0, s>>>(nc_i, raw_start_.p, raw_j_.p, keep_.p, (int)tile_cap_,
                                            tile_start_.p, anc_.p, ext_.p, bd, box_, wrap_pad(), tile_i_.p,
                                            tile_j_.p, tile_mask_.p, tile_shift_.p);
    const int nnz = (int)cs.ex_j.size();
    OCM_CK(cudaMemsetAsync(mask_count_.p, 0, sizeof(int32_t), s));
    if (nnz > 0) {
        k_excl<false><<<div_up(nnz, 256), 256, 0, s>>>(nnz, nc_i, (int)tile_cap_, ex_start_.p, ex_j_.p, ex_bits_.p, slot_.p,
                                                        tile_start_.p, tile_j_.p, tile_mask_.p,
                                                        masks_.p, mask_count_.p, (int)mask_cap_,
                                                        flags_.p);
        k_excl<true><<<div_up(nnz, 256), 256, 0, s>>>(nnz, nc_i, (int)tile_cap_, ex_start_.p, ex_j_.p, ex_bits_.p, slot_.p,
                                                       tile_start_.p, tile_j_.p, tile_mask_.p,
                                                       masks_.p, mask_count_.p, (int)mask_cap_,
                                                       flags_.p);
    }
    OCM_CK(cudaGetLastError());
    if (charged_split_) {
        // cell sort done with the beads' (the split implies the reordered layout)
        const int m = (int)n_charged_;
        const float ccut = (float)(std::sqrt((double)cs.pc.dh_rc2) + skin) * 1.0001f + 1e-4f;
        k_chg_rows<<<div_up((int64_t)m * 32, 128), 128, 0, s>>>(
            m, chg_idx_.p, chg_key_.p, xq_.p, charged_cells_[0], charged_cells_[1], charged_cells_[2], box_,
            inv_box_, ccut * ccut, chg_start_.p, chg_sorted_.p, ex_csr_.p, ex_j_.p, ex_bits_.p, chg_rows_.p,
            chg_len_.p, (int)chg_row_cap_, chg_stats_.p, flags_.p);
    }
}

void PlainContext::launch_forces(cudaStream_t s, bool energy, uint32_t slots_enabled, int) {
    ForceArgs a{};
    a.nc = (int)nc;
    a.tile_cap = (int)tile_cap_;
    a.n = (int)n;
    // enough warps for every chunk of the largest list the buffers hold,
    // capped at 32 resident blocks per SM (the loop strides over the rest)
    a.blocks_tiles = (int)std::max<int64_t>(
        1, std::min<int64_t>(div_up(tile_cap_, kTilesPerChunk * kWarpsPerForceBlock), 32 * (int64_t)num_sms_));
    a.n_bonds = (int)cs.bonds.size();
    a.n_angles = (int)cs.angles.size();
    a.n_dih = (int)cs.dihedrals.size();
    a.blocks_bonds = div_up(a.n_bonds, kForceThreads);
    a.blocks_angles = div_up(a.n_angles, kForceThreads);
    a.blocks_dih = div_up(a.n_dih, kForceThreads);
    a.xs = xs_.p; a.p0s = p0s_.p; a.p1s = p1s_.p; a.labs = labs_.p; a.perm = perm_.p;
    a.tile_start = tile_start_.p; a.tile_i = tile_i_.p; a.tile_j = tile_j_.p; a.tile_mask = tile_mask_.p;
    a.masks = masks_.p;
    a.x = x_.p; a.y = y_.p; a.z = z_.p;
    a.bonds = bonds_.p; a.angles = angles_.p; a.fla = fla_.p; a.dih = dihedrals_.p; a.fld = fld_.p;
    a.F = F_.p;
    a.pc = cs.pc;
    a.box = box_;
    a.inv_box = inv_box_;
    a.slots_enabled = slots_enabled;
    uint32_t excl_all = 0;
    const int pair_slots[4] = {kSlotEXV, kSlotDH, kSlotLJR, kSlotLJA};
    for (int t = 0; t < 4; ++t)
        if (!(slots_enabled & (1u << pair_slots[t]))) excl_all |= 1u << t;
    if (charged_split_) {
        // the tiles leave Debye-Hueckel to the charged-pair list
        excl_all |= kTermDH;
        a.pc.list_rc2 = (float)(tile_cutoff_ * tile_cutoff_);
    }
    a.excl_all = excl_all;
    a.xq = xq_.p;
    a.xlo = xlo_.p;
    a.p0 = p0_.p;
    a.tile_shift = tile_shift_.p;
    a.chg_idx = chg_idx_.p;
    a.chg_rows = chg_rows_.p;
    a.chg_len = chg_len_.p;
    a.n_chg = (int)n_charged_;
    a.chg_row_cap = (int)chg_row_cap_;
    a.flags = flags_.p;
    a.blocks_chg = charged_split_ ? (int)std::max<int64_t>(1, div_up(n_charged_, kWarpsPerForceBlock)) : 0;
    a.energy = energy_.p;
    int blocks_tiles = a.blocks_tiles;
    if ((cs.pc.terms & ~excl_all & 15) == 0) {
        a.blocks_tiles = 0;
        blocks_tiles = 0;
    }
    const int grid = blocks_tiles + a.blocks_bonds + a.blocks_angles + a.blocks_dih + a.blocks_chg;
    if (grid == 0) return;
    // the tiles' pair terms (Debye-Hueckel leaves them for the charged rows)
    const int terms = cs.pc.terms & ~(charged_split_ ? kTermDH : 0);
    const bool per = cs.periodic;
    if ((terms & ~(kTermEXV | kTermDH)) == 0) launch_forces_t<kTermEXV | kTermDH>(a, grid, s, per, energy);
    else if (terms == (kTermLJR | kTermLJA) && cs.lj_same_sigma)
        launch_forces_t<kTermLJR | kTermLJA | kLJSameSigma>(a, grid, s, per, energy);
    else if ((terms & ~(kTermLJR | kTermLJA)) == 0) launch_forces_t<kTermLJR | kTermLJA>(a, grid, s, per, energy);
    else if ((terms & ~(kTermLJR | kTermLJA | kTermDH)) == 0)
        launch_forces_t<kTermLJR | kTermLJA | kTermDH>(a, grid, s, per, energy);
    else launch_forces_t<15>(a, grid, s, per, energy);
    OCM_CK(cudaGetLastError());
}

void PlainContext::launch_integrate(cudaStream_t s, int r) {
    IntegrateArgs a{};
    a.n = (int)n;
    a.F = F_.p;
    a.vx = vx_.p; a.vy = vy_.p; a.vz = vz_.p;
    a.x = x_.p; a.y = y_.p; a.z = z_.p;
    a.invm = invm_.p;
    a.xq = xq_.p; a.xlo = xlo_.p; a.xs = xs_.p; a.anc = anc_.p; a.slot = slot_.p; a.ref = ref_.p;
    a.lc = lc_;
    a.step_base = step_base_.p;
    a.r = r;
    a.periodic = cs.periodic ? 1 : 0;
    for (int k = 0; k < 3; ++k) {
        a.box[k] = cs.box[k];
        a.inv_box[k] = cs.box[k] > 0 ? 1.0 / cs.box[k] : 0.0;
    }
    a.fbox = box_;
    a.finv_box = inv_box_;
    const float half = (float)(0.5 * skin);
    a.disp_limit2 = half * half;
    a.flags = flags_.p;
    k_integrate<<<div_up(n, 64), 64, 0, s>>>(a);  // small blocks: every SM gets some
    OCM_CK(cudaGetLastError());
}

void PlainContext::ensure_capacity() {
    // Build once eagerly, read the sizes back and grow the buffers if needed.
    for (int attempt = 0; attempt < 8; ++attempt) {
        OCM_CK(cudaMemsetAsync(flags_.p, 0, sizeof(int32_t), stream_));
        rebuild(stream_);
        int32_t total = 0, masks = 0, flags = 0, chg[2] = {0, 0};
        if (charged_split_)
            OCM_CK(cudaMemcpyAsync(chg, chg_stats_.p, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost, stream_));
        int32_t kept = 0;  // tiles after pruning
        OCM_CK(cudaMemcpyAsync(&total, raw_start_.p + nc, sizeof(int32_t), cudaMemcpyDeviceToHost, stream_));
        OCM_CK(cudaMemcpyAsync(&kept, tile_start_.p + nc, sizeof(int32_t), cudaMemcpyDeviceToHost, stream_));
        OCM_CK(cudaMemcpyAsync(&masks, mask_count_.p, sizeof(int32_t), cudaMemcpyDeviceToHost, stream_));
        OCM_CK(cudaMemcpyAsync(&flags, flags_.p, sizeof(int32_t), cudaMemcpyDeviceToHost, stream_));
        OCM_CK(cudaStreamSynchronize(stream_));
        // A buffer that is reallocated loses the list just built into it, so
        // any growth (also the pre-emptive one below 80% headroom) is
        // followed by another build before the list is used.
        bool realloced = false;
        if (total > tile_cap_ || (int64_t)total * 5 / 4 + 64 > tile_cap_) {
            const int64_t want = std::min<int64_t>(nc * (nc + 1) / 2, (int64_t)total * 2 + 1024);
            if (want > tile_cap_) {
                tile_cap_ = want;
                alloc_tile_arrays();
                realloced = true;
                clear_graphs();
            }
        }
        if (masks > mask_cap_ || (int64_t)masks * 5 / 4 + 16 > mask_cap_) {
            const int64_t want = std::min<int64_t>(tile_cap_, (int64_t)masks * 2 + 256);
            if (want > mask_cap_) {
                mask_cap_ = want;
                masks_.alloc(mask_cap_ * 128);
                realloced = true;
                clear_graphs();
            }
        }
        if (charged_split_ && ((int64_t)chg[0] * 5 / 4 + 16 > chg_row_cap_)) {
            // rows with 25% headroom, a multiple of 32 entries
            const int64_t want = ((int64_t)chg[0] * 3 / 2 + 32 + 31) / 32 * 32;
            if (want > chg_row_cap_) {
                chg_row_cap_ = want;
                chg_rows_.alloc(n_charged_ * chg_row_cap_);
                realloced = true;
                clear_graphs();
            }
        }
        if (!realloced &&
            !(flags & (ListFlags::kTileOverflow | ListFlags::kMaskOverflow | ListFlags::kChargedOverflow)) &&
            total <= tile_cap_ && masks <= mask_cap_ && chg[0] <= chg_row_cap_) {
            tiles_last = kept;
            masked_last = masks;
            charged_last_ = chg[1] / 2;
            list_builds++;
            return;
        }
    }
    throw Error(4, "[error] tile list capacity could not be established");
}

uint32_t PlainContext::slots_for_groups(uint32_t groups) const {
    uint32_t s = 0;
    for (int k = 0; k < kNumSlots; ++k)
        if (cs.slot_group[k] >= 0 && (groups >> cs.slot_group[k]) & 1u) s |= 1u << k;
    return s;
}

// Returns true when the evaluation flagged a blown-up system (the outputs
// are filled all the same).
bool PlainContext::eval(uint32_t groups, bool energy, double* forces, double* slot_energy) {
    OCM_CK(cudaSetDevice(device));
    check_positions_set();
    ensure_capacity();
    OCM_CK(cudaMemsetAsync(energy_.p, 0, kNumSlots * sizeof(double), stream_));
    OCM_CK(cudaMemsetAsync(F_.p, 0, 3 * n * sizeof(unsigned long long), stream_));
    OCM_CK(cudaMemsetAsync(flags_.p, 0, sizeof(int32_t), stream_));
    launch_forces(stream_, energy, slots_for_groups(groups), 0);
    int32_t flags = 0;
    OCM_CK(cudaMemcpyAsync(&flags, flags_.p, sizeof(int32_t), cudaMemcpyDeviceToHost, stream_));
    std::vector<unsigned long long> f;
    if (forces) {
        f.resize(3 * n);
        OCM_CK(cudaMemcpyAsync(f.data(), F_.p, 3 * n * sizeof(unsigned long long),
                               cudaMemcpyDeviceToHost, stream_));
    }
    double e[kNumSlots];
    OCM_CK(cudaMemcpyAsync(e, energy_.p, sizeof(e), cudaMemcpyDeviceToHost, stream_));
    OCM_CK(cudaMemsetAsync(F_.p, 0, 3 * n * sizeof(unsigned long long), stream_));
    OCM_CK(cudaStreamSynchronize(stream_));
    if (forces)
        for (int64_t i = 0; i < n; ++i)
            for (int c = 0; c < 3; ++c)
                forces[3 * i + c] = (double)(long long)f[c * n + i] * kFixedInv;
    if (slot_energy)
        for (int k = 0; k < kNumSlots; ++k) slot_energy[k] = e[k];
    return (flags & ListFlags::kBlownUp) != 0;
}

static void throw_blown_up() {
    throw Error(7, "[error] non-finite force, or a force of 1e9 kJ/mol/nm or more (outputs filled)");
}

void PlainContext::get_state(uint32_t groups, double* forces, double* energy) {
    double se[kNumSlots];
    const bool blown = eval(groups, energy != nullptr, forces, se);
    if (energy) {
        double tot = 0;
        for (int k = 0; k < kNumSlots; ++k)
            if (cs.slot_group[k] >= 0 && ((groups >> cs.slot_group[k]) & 1u)) tot += se[k];
        *energy = tot;
    }
    if (blown) throw_blown_up();
}

void PlainContext::group_energies(double* e32) {
    double se[kNumSlots];
    const bool blown = eval(0xffffffffu, true, nullptr, se);
    for (int g = 0; g < 32; ++g) e32[g] = 0.0;
    for (int k = 0; k < kNumSlots; ++k)
        if (cs.slot_group[k] >= 0) e32[cs.slot_group[k]] += se[k];
    if (blown) throw_blown_up();
}

cudaGraphExec_t PlainContext::graph_for(int chunk) {
    auto it = graphs_.find(chunk);
    if (it != graphs_.end()) return it->second;
    cudaGraph_t g;
    OCM_CK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    try {
        rebuild(stream_);
        const uint32_t all = slots_for_groups(0xffffffffu);
        for (int r = 0; r < chunk; ++r) {
            launch_forces(stream_, false, all, r);
            launch_integrate(stream_, r);
        }
        k_advance<<<1, 1, 0, stream_>>>(step_base_.p, (unsigned long long)chunk);
    } catch (...) {
        cudaStreamEndCapture(stream_, &g);
        throw;
    }
    OCM_CK(cudaStreamEndCapture(stream_, &g));
    cudaGraphExec_t exec;
    OCM_CK(cudaGraphInstantiate(&exec, g, 0));
    cudaGraphDestroy(g);
    graphs_[chunk] = exec;
    return exec;
}

void PlainContext::set_engine(int32_t mode) {
    if (mode != kEngineAuto && mode != kEngineTiles && mode != kEngineOneSystem)
        throw Error(1, "[error] engine must be 0 (auto), 1 (tiles) or 2 (one-system batched kernel)");
    if (mode == kEngineOneSystem && (cs.periodic || n > 2048))
        throw Error(6, "[error] the one-system batched kernel runs non-periodic systems of at most 2048 beads");
    engine_mode_ = mode;
}

bool PlainContext::one_system_eligible() {
    if (engine_mode_ == kEngineTiles || one_refused_) return false;
    if (cs.periodic) return false;
    for (const auto& b : cs.bonds)
        if (b.periodic) return false;
    return engine_mode_ == kEngineOneSystem || n <= kOneSystemMaxBeads;
}

// step() on the batched kernel as a one-system persistent launch: the
// context's positions, velocities and step counter go device-to-device into
// a one-slot batch, which runs the steps in shared memory on one SM, and
// come back.  The Langevin noise is the same counter-based stream (seed,
// bead, step) as on the tiles, so the physics is the same and only FP32
// rounding differs.  The first call builds the batch (a host copy of the
// state for the admission); a system the batched kernel does not take goes
// to the tiles from then on.
void PlainContext::step_one_system(int64_t nsteps) {
    OCM_CK(cudaStreamSynchronize(stream_));
    if (!one_) {
        std::vector<double> x(3 * n), v(3 * n);
        get_positions(x.data());
        get_velocities(v.data());
        const int64_t fp = BatchEngine::footprint(desc_);
        const int64_t arena = std::max<int64_t>(n, fp / 256 + 64);
        auto b = std::make_unique<BatchEngine>(device, 1, arena, (int32_t)n);
        one_slot_ = b->admit(desc_, x.data(), v.data(), one_T_, one_friction_, one_dt_, one_seed_, 0, 0);
        one_ = std::move(b);
    }
    unsigned long long base = 0;
    OCM_CK(cudaMemcpy(&base, step_base_.p, sizeof(base), cudaMemcpyDeviceToHost));
    one_->load_state_device(one_slot_, x_.p, y_.p, z_.p, vx_.p, vy_.p, vz_.p, base, base + (uint64_t)nsteps);
    for (int64_t left = nsteps; left > 0;) {
        const int32_t chunk = (int32_t)std::min<int64_t>(left, 4096);
        one_->run(chunk, false);
        left -= chunk;
    }
    if (one_->slot_status(one_slot_) != 0)
        throw Error(7, "[error] the system blew up (a non-finite force, velocity or position, or a force of "
                       "1e9 kJ/mol/nm or more); the context keeps its state from before this step call");
    one_->store_state_device(one_slot_, x_.p, y_.p, z_.p, vx_.p, vy_.p, vz_.p);
    k_advance<<<1, 1, 0, stream_>>>(step_base_.p, (unsigned long long)nsteps);
    OCM_CK(cudaGetLastError());
    k_positions_to_float<<<div_up(n, 256), 256, 0, stream_>>>(
        (int)n, x_.p, y_.p, z_.p, 0, cs.box[0], cs.box[1], cs.box[2], 0.0, 0.0, 0.0, xq_.p, xlo_.p);
    OCM_CK(cudaGetLastError());
    OCM_CK(cudaStreamSynchronize(stream_));
    steps_done += nsteps;
    last_step_one_system_ = true;
}

void PlainContext::step(int64_t nsteps) {
    OCM_CK(cudaSetDevice(device));
    check_positions_set();
    if (nsteps < 0) throw Error(1, "[error] negative step count");
    if (nsteps == 0) return;
    if (one_system_eligible()) {
        try {
            step_one_system(nsteps);
            return;
        } catch (const Error& e) {
            // a system the batched kernel does not take (shared memory,
            // list capacity) runs on the tiles; other errors propagate
            if (one_ || (e.code != 3 && e.code != 6) || engine_mode_ == kEngineOneSystem) throw;
            one_refused_ = true;
        }
    }
    last_step_one_system_ = false;
    if (graphs_.empty()) ensure_capacity();
    for (int attempt = 0; attempt < 12; ++attempt) {
        cudaStream_t s = stream_;
        OCM_CK(cudaMemcpyAsync(sx_.p, x_.p, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        OCM_CK(cudaMemcpyAsync(sy_.p, y_.p, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        OCM_CK(cudaMemcpyAsync(sz_.p, z_.p, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        OCM_CK(cudaMemcpyAsync(svx_.p, vx_.p, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
        OCM_CK(cudaMemcpyAsync(svy_.p, vy_.p, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
        OCM_CK(cudaMemcpyAsync(svz_.p, vz_.p, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
        OCM_CK(cudaMemcpyAsync(sstep_.p, step_base_.p, sizeof(unsigned long long),
                               cudaMemcpyDeviceToDevice, s));
        OCM_CK(cudaMemsetAsync(flags_.p, 0, sizeof(int32_t), s));
        int64_t left = nsteps;
        int64_t launches = 0;
        while (left > 0) {
            const int chunk = (int)std::min<int64_t>(left, rebuild_interval);
            OCM_CK(cudaGraphLaunch(graph_for(chunk), s));
            left -= chunk;
            launches++;
        }
        OCM_CK(cudaMemcpyAsync(h_flags_, flags_.p, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        OCM_CK(cudaStreamSynchronize(s));
        const int32_t flags = h_flags_[0];
        if (flags == 0) {
            steps_done += nsteps;
            list_builds += launches;
            return;
        }
        // restore and retry with more capacity / more frequent rebuilds
        OCM_CK(cudaMemcpyAsync(x_.p, sx_.p, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        OCM_CK(cudaMemcpyAsync(y_.p, sy_.p, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        OCM_CK(cudaMemcpyAsync(z_.p, sz_.p, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        OCM_CK(cudaMemcpyAsync(vx_.p, svx_.p, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
        OCM_CK(cudaMemcpyAsync(vy_.p, svy_.p, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
        OCM_CK(cudaMemcpyAsync(vz_.p, svz_.p, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
        OCM_CK(cudaMemcpyAsync(step_base_.p, sstep_.p, sizeof(unsigned long long),
                               cudaMemcpyDeviceToDevice, s));
        OCM_CK(cudaMemsetAsync(F_.p, 0, 3 * n * sizeof(unsigned long long), s));
        k_positions_to_float<<<div_up(n, 256), 256, 0, s>>>(
            (int)n, x_.p, y_.p, z_.p, cs.periodic ? 1 : 0, cs.box[0], cs.box[1], cs.box[2],
            cs.box[0] > 0 ? 1.0 / cs.box[0] : 0.0, cs.box[1] > 0 ? 1.0 / cs.box[1] : 0.0,
            cs.box[2] > 0 ? 1.0 / cs.box[2] : 0.0, xq_.p, xlo_.p);
        OCM_CK(cudaStreamSynchronize(s));
        if (flags & ListFlags::kBlownUp)
            throw Error(7, "[error] the system blew up (a non-finite force, velocity or position, or a force of "
                           "1e9 kJ/mol/nm or more); the context keeps its state from before this step call");
        if (flags & ListFlags::kSkinViolation) {
            if (rebuild_interval == 1)
                throw Error(7, "[error] particles moved more than half the skin in one step");
            rebuild_interval = std::max(1, rebuild_interval / 2);
        }
        if (flags & ListFlags::kChargedOverflow) {
            chg_row_cap_ *= 2;
            chg_rows_.alloc(n_charged_ * chg_row_cap_);
        }
        if (flags & (ListFlags::kTileOverflow | ListFlags::kMaskOverflow)) {
            tile_cap_ = std::min<int64_t>(nc * (nc + 1) / 2, tile_cap_ * 2);
            alloc_tile_arrays();
            mask_cap_ = std::min<int64_t>(tile_cap_, mask_cap_ * 2);
            masks_.alloc(mask_cap_ * 128);
        }
        clear_graphs();
        ensure_capacity();
    }
    throw Error(4, "[error] step could not complete after repeated list rebuilds");
}

void PlainContext::set_list_options(int32_t interval, double sk) {
    if (interval < 0 || sk < 0) throw Error(1, "[error] invalid list options");
    if (interval > 0) rebuild_interval = interval;
    if (sk > 0) skin = sk;
    setup_charged_cells();  // cells must stay at least cutoff + skin wide
    clear_graphs();
}

// Every per-tile array, at tile_cap_ entries (candidate and final lists).
void PlainContext::alloc_tile_arrays() {
    tile_i_.alloc(tile_cap_);
    tile_j_.alloc(tile_cap_);
    tile_mask_.alloc(tile_cap_);
    tile_shift_.alloc(tile_cap_);
    raw_i_.alloc(tile_cap_);
    raw_j_.alloc(tile_cap_);
    keep_.alloc(tile_cap_);
}

float PlainContext::wrap_pad() const {
    // two beads' displacement allowance between builds, plus rounding
    return (float)(skin * 1.001 + 1e-3);
}

BoxD PlainContext::box_d() const {
    BoxD b{};
    for (int k = 0; k < 3; ++k) {
        b.L[k] = cs.box[k];
        b.iL[k] = cs.box[k] > 0 ? 1.0 / cs.box[k] : 0.0;
    }
    b.periodic = cs.periodic ? 1 : 0;
    return b;
}

void PlainContext::setup_columns(double width) {
    // Columns of about `width` in x and y, z slices of 0.25 nm (fewer when
    // the cells would outnumber the beads four to one).
    width = std::max(width, col_wmin_);
    int dims[3];
    for (int a = 0; a < 2; ++a) dims[a] = (int)std::max(1.0, std::min(1023.0, std::floor(cs.box[a] / width)));
    const int64_t ncols = (int64_t)dims[0] * dims[1];
    const int64_t zmax = std::max<int64_t>(1, std::max<int64_t>(4 * n, 65536) / ncols);
    dims[2] = (int)std::max<int64_t>(1, std::min<int64_t>(zmax, (int64_t)std::floor(cs.box[2] / 0.25)));
    if (dims[0] == cell_dims_[0] && dims[1] == cell_dims_[1] && dims[2] == cell_dims_[2] && n_cells_ > 0) return;
    for (int a = 0; a < 3; ++a) cell_dims_[a] = dims[a];
    n_cells_ = ncols * dims[2];
    cell_count_.alloc(n_cells_);
    cell_start_.alloc(n_cells_ + 1);
    cell_fill_.alloc(n_cells_);
    col_start_.alloc(ncols + 1);
    clear_graphs();
}

void PlainContext::setup_charged_cells() {
    if (!charged_split_) return;
    const double cell = (std::sqrt((double)cs.pc.dh_rc2) + skin) * 1.0001 + 1e-4;
    int dims[3];
    for (int a = 0; a < 3; ++a) dims[a] = (int)std::min(1023.0, std::floor(cs.box[a] / cell));
    if (dims[0] < 3 || dims[1] < 3 || dims[2] < 3) {
        // box too narrow for a 27-cell neighbourhood: back to one tile list
        charged_split_ = false;
        tile_cutoff_ = cs.max_cutoff;
        clear_graphs();
        return;
    }
    for (int a = 0; a < 3; ++a) charged_cells_[a] = dims[a];
    n_charged_cells_ = (int64_t)dims[0] * dims[1] * dims[2];
    chg_count_.alloc(n_charged_cells_);
    chg_start_.alloc(n_charged_cells_ + 1);
    chg_fill_.alloc(n_charged_cells_);
    clear_graphs();
}

void PlainContext::list_pairs(int64_t* out, int64_t cap, int64_t* n_out) {
    OCM_CK(cudaSetDevice(device));
    check_positions_set();
    ensure_capacity();
    DevBuf<long long> buf;
    buf.alloc(std::max<int64_t>(1, 2 * cap));
    DevBuf<unsigned long long> cnt;
    cnt.alloc(1);
    OCM_CK(cudaMemsetAsync(cnt.p, 0, sizeof(unsigned long long), stream_));
    const int wblocks = div_up(nc * 32, 128);
    const float tile_rc2 = charged_split_ ? (float)(tile_cutoff_ * tile_cutoff_) : cs.pc.list_rc2;
    if (cs.periodic)
        k_list_pairs<true><<<wblocks, 128, 0, stream_>>>((int)nc, xs_.p, tile_shift_.p, perm_.p, tile_start_.p,
                                                        tile_j_.p, box_, inv_box_, tile_rc2,
                                                        buf.p, cap, cnt.p, tile_cap_);
    else
        k_list_pairs<false><<<wblocks, 128, 0, stream_>>>((int)nc, xs_.p, tile_shift_.p, perm_.p, tile_start_.p,
                                                         tile_j_.p, box_, inv_box_, tile_rc2,
                                                         buf.p, cap, cnt.p, tile_cap_);
    if (charged_split_)
        k_chg_list_pairs<<<(int)n_charged_, 128, 0, stream_>>>(
            (int)n_charged_, chg_idx_.p, chg_rows_.p, chg_len_.p, (int)chg_row_cap_, xq_.p, xlo_.p, box_, inv_box_,
            cs.pc.dh_rc2, buf.p, cap,
            cnt.p);
    OCM_CK(cudaGetLastError());
    unsigned long long c = 0;
    OCM_CK(cudaMemcpyAsync(&c, cnt.p, sizeof(c), cudaMemcpyDeviceToHost, stream_));
    OCM_CK(cudaStreamSynchronize(stream_));
    *n_out = (int64_t)c;
    if ((int64_t)c > cap) throw Error(1, "[error] output capacity too small");
    OCM_CK(cudaMemcpy(out, buf.p, 2 * c * sizeof(long long), cudaMemcpyDeviceToHost));
}

void PlainContext::cluster_order(int64_t* out, int64_t cap, int64_t* n_out) {
    OCM_CK(cudaSetDevice(device));
    check_positions_set();
    ensure_capacity();
    *n_out = np;
    if (cap < np) throw Error(1, "[error] output capacity too small");
    std::vector<int32_t> p(np);
    OCM_CK(cudaMemcpy(p.data(), perm_.p, np * sizeof(int32_t), cudaMemcpyDeviceToHost));
    for (int64_t k = 0; k < np; ++k) out[k] = p[k];
}

}  // namespace ocm
