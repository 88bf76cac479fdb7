// bvh_build.cu — GPU LBVH build. Replaces the driver-side BLAS/TLAS builds of
// the reference (src/ray/acceleration.rs:44-126, 135-239, 344-400), which
// have no source: on GB300 there are no RT cores, so the hierarchy is built
// here from the triangles of the flattened scene.
//
// Pipeline (all on the context stream):
//   1. centroids + centroid bounds (block reduction, ordered-int atomics)
//   2. 30-bit Morton codes of centroids in cubic cells over the centroid
//      bounds (all axes scaled by the largest extent)
//   3. stable LSD radix sort of (code, triangle) with 8-bit digits
//   4. Karras 2012 radix-tree hierarchy over the sorted codes, equal codes
//      split by index (delta = 32 + clz(i ^ j))
//   5. bottom-up refit with one arrival flag per node; the second child to
//      arrive computes the parent box
//   6. triangle stream in leaf order (48 B per triangle)
// Min/max are order-independent and the sort is stable, so the topology and
// every box are a pure function of the input: they equal the CPU LBVH of the
// oracle bit for bit.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

#include "bvh8.cuh"
#include "bvh8_traverse.cuh"
#include "internal.h"

namespace solrt {

namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;

__device__ __forceinline__ unsigned int float_to_ordered(float f) {
    const unsigned int b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float ordered_to_float(unsigned int o) {
    return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
}

// centroid = ((p0 + p1) + p2) / 3 per axis; bounds as ordered ints.
__global__ void k_centroids(const float4* __restrict__ vpos, const uint4* __restrict__ tri_idx, uint32_t n,
                            float4* __restrict__ cen, unsigned int* __restrict__ cb) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float c[3] = {INFINITY, INFINITY, INFINITY};
    float mn[3], mx[3];
    if (i < n) {
        const uint4 t = tri_idx[i];
        const float4 a = vpos[t.x], b = vpos[t.y], d = vpos[t.z];
        c[0] = ((a.x + b.x) + d.x) / 3.0f;
        c[1] = ((a.y + b.y) + d.y) / 3.0f;
        c[2] = ((a.z + b.z) + d.z) / 3.0f;
        cen[i] = make_float4(c[0], c[1], c[2], 0.0f);
        for (int k = 0; k < 3; ++k) { mn[k] = c[k]; mx[k] = c[k]; }
    } else {
        for (int k = 0; k < 3; ++k) { mn[k] = INFINITY; mx[k] = -INFINITY; }
    }
    for (int k = 0; k < 3; ++k) {
        for (int off = 16; off > 0; off >>= 1) {
            mn[k] = fminf(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], off));
            mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], off));
        }
    }
    // one atomic per block and bound (per-warp atomics on six addresses
    // serialise at millions of triangles)
    __shared__ float s_mn[3][32], s_mx[3][32];
    const int warp = threadIdx.x >> 5, nwarps = (blockDim.x + 31) >> 5;
    if ((threadIdx.x & 31) == 0) {
        for (int k = 0; k < 3; ++k) {
            s_mn[k][warp] = mn[k];
            s_mx[k][warp] = mx[k];
        }
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        const int k = threadIdx.x;
        float a = s_mn[k][0], b = s_mx[k][0];
        for (int w = 1; w < nwarps; ++w) {
            a = fminf(a, s_mn[k][w]);
            b = fmaxf(b, s_mx[k][w]);
        }
        atomicMin(cb + k, float_to_ordered(a));
        atomicMax(cb + 3 + k, float_to_ordered(b));
    }
}

__device__ __forceinline__ uint32_t expand_bits10(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__device__ __forceinline__ uint32_t quantise10(float c, float lo, float ext) {
    if (!(ext > 0.0f)) return 0;
    const float f = ((c - lo) / ext) * 1024.0f;
    if (f >= 1023.0f) return 1023;
    if (!(f > 0.0f)) return 0;
    return (uint32_t)f;
}

__global__ void k_morton(const float4* __restrict__ cen, const unsigned int* __restrict__ cb, uint32_t n,
                         uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float lo[3] = {ordered_to_float(cb[0]), ordered_to_float(cb[1]), ordered_to_float(cb[2])};
    const float hi[3] = {ordered_to_float(cb[3]), ordered_to_float(cb[4]), ordered_to_float(cb[5])};
    const float4 c = cen[i];
    // cubic cells: every axis is scaled by the largest extent, so a long
    // thin scene does not get cells stretched along its long axis
    const float ext = fmaxf(fmaxf(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
    const uint32_t qx = quantise10(c.x, lo[0], ext);
    const uint32_t qy = quantise10(c.y, lo[1], ext);
    const uint32_t qz = quantise10(c.z, lo[2], ext);
    keys[i] = (expand_bits10(qx) << 2) | (expand_bits10(qy) << 1) | expand_bits10(qz);
    vals[i] = i;
}

// ---- stable LSD radix sort, 8-bit digits -------------------------------------
// Tile = 2048 keys per block, read in 8 rounds of 256 (item = r*256 + t).

__global__ void __launch_bounds__(kSortThreads) k_radix_hist(const uint32_t* __restrict__ keys, uint32_t n,
                                                             int shift, uint32_t nblocks,
                                                             uint32_t* __restrict__ hist) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * kSortTile;
    for (int r = 0; r < kSortItems; ++r) {
        const uint32_t idx = base + r * kSortThreads + threadIdx.x;
        if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of `len` counts with one block of 1024 threads.
__global__ void __launch_bounds__(1024) k_scan_exclusive(uint32_t* __restrict__ data, uint32_t len) {
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t base = 0; base < len; base += 1024) {
        const uint32_t idx = base + threadIdx.x;
        const uint32_t v = idx < len ? data[idx] : 0u;
        uint32_t x = v;
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= off) x += y;
        }
        if (lane == 31) warp_sums[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = warp_sums[lane];
            for (int off = 1; off < 32; off <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, w, off);
                if (lane >= off) w += y;
            }
            warp_sums[lane] = w;
        }
        __syncthreads();
        const uint32_t incl = x + (warp > 0 ? warp_sums[warp - 1] : 0u) + carry;
        if (idx < len) data[idx] = incl - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry = incl;
        __syncthreads();
    }
}

// Exclusive scan of a long array in three launches: per-tile sums (tiles of
// kScanTile counts, 4 per thread), one-block scan of the tile sums, then each
// tile's scan offset by its tile's sum.
constexpr int kScanTile = 4096;

__device__ __forceinline__ uint32_t block_exclusive_1024(uint32_t x, uint32_t* warp_sums, uint32_t* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = x;
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += y;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = warp_sums[lane];
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, off);
            if (lane >= off) w += y;
        }
        warp_sums[lane] = w;
    }
    __syncthreads();
    if (total) *total = warp_sums[31];
    return incl - x + (warp > 0 ? warp_sums[warp - 1] : 0u);
}

__global__ void __launch_bounds__(1024) k_scan_reduce(const uint32_t* __restrict__ data, uint32_t len,
                                                      uint32_t* __restrict__ sums) {
    __shared__ uint32_t warp_sums[32];
    const uint32_t base = blockIdx.x * kScanTile + 4u * threadIdx.x;
    uint32_t x = 0;
    for (uint32_t i = 0; i < 4; ++i)
        if (base + i < len) x += data[base + i];
    uint32_t total = 0;
    block_exclusive_1024(x, warp_sums, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) k_scan_apply(uint32_t* __restrict__ data, uint32_t len,
                                                     const uint32_t* __restrict__ sums) {
    __shared__ uint32_t warp_sums[32];
    const uint32_t base = blockIdx.x * kScanTile + 4u * threadIdx.x;
    uint32_t v[4];
    uint32_t x = 0;
    for (uint32_t i = 0; i < 4; ++i) {
        v[i] = base + i < len ? data[base + i] : 0u;
        x += v[i];
    }
    uint32_t run = block_exclusive_1024(x, warp_sums, nullptr) + sums[blockIdx.x];
    for (uint32_t i = 0; i < 4; ++i) {
        if (base + i < len) data[base + i] = run;
        run += v[i];
    }
}

__global__ void __launch_bounds__(kSortThreads) k_radix_scatter(const uint32_t* __restrict__ kin,
                                                                const uint32_t* __restrict__ vin,
                                                                uint32_t* __restrict__ kout,
                                                                uint32_t* __restrict__ vout,
                                                                const uint32_t* __restrict__ scan, uint32_t n,
                                                                int shift, uint32_t nblocks) {
    __shared__ uint32_t base[256];
    __shared__ uint32_t wcount[kSortThreads / 32][256];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    base[t] = scan[t * nblocks + blockIdx.x];
    const uint32_t lane_lt = (1u << lane) - 1u;
    const uint32_t tile = blockIdx.x * kSortTile;
    for (int r = 0; r < kSortItems; ++r) {
        for (int d = lane; d < 256; d += 32) wcount[warp][d] = 0;
        __syncthreads();
        const uint32_t idx = tile + r * kSortThreads + t;
        const bool valid = idx < n;
        const uint32_t key = valid ? kin[idx] : 0u;
        const uint32_t digit = valid ? ((key >> shift) & 255u) : 256u;
        const uint32_t peers = __match_any_sync(0xffffffffu, digit);
        const uint32_t rank = __popc(peers & lane_lt);
        if (valid && rank == 0) wcount[warp][digit] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t off = base[digit] + rank;
            for (int w = 0; w < warp; ++w) off += wcount[w][digit];
            if (off < n) {
                kout[off] = key;
                vout[off] = vin[idx];
            }
        }
        __syncthreads();
        uint32_t tot = 0;
        for (int w = 0; w < kSortThreads / 32; ++w) tot += wcount[w][t];
        base[t] += tot;
        __syncthreads();
    }
}

// ---- Karras hierarchy ------------------------------------------------------

__device__ __forceinline__ int kdelta(const uint32_t* __restrict__ k, int64_t n, int64_t i, int64_t j) {
    if (j < 0 || j > n - 1) return -1;
    const uint32_t a = k[i], b = k[j];
    if (a == b) return 32 + __clz((uint32_t)i ^ (uint32_t)j);
    return __clz(a ^ b);
}

// child[2i], child[2i+1]: internal index, or 0x80000000 | leaf position.
// range[i] (optional): first and last leaf position under internal node i.
__global__ void k_karras(const uint32_t* __restrict__ keys, uint32_t n, uint32_t* __restrict__ child,
                         uint32_t* __restrict__ parent_int, uint32_t* __restrict__ parent_leaf,
                         uint2* __restrict__ range) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= (int64_t)n - 1) return;
    const int d = (kdelta(keys, n, i, i + 1) - kdelta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = kdelta(keys, n, i, i - d);
    int64_t lmax = 2;
    while (kdelta(keys, n, i, i + lmax * d) > dmin) lmax *= 2;
    int64_t l = 0;
    for (int64_t t = lmax / 2; t >= 1; t /= 2)
        if (kdelta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    const int64_t j = i + l * d;
    const int dnode = kdelta(keys, n, i, j);
    int64_t s = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (kdelta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int64_t g = i + s * d + (d < 0 ? d : 0);
    const int64_t lo = i < j ? i : j, hi = i < j ? j : i;
    uint32_t left, right;
    if (lo == g) { left = 0x80000000u | (uint32_t)g; parent_leaf[g] = (uint32_t)i; }
    else { left = (uint32_t)g; parent_int[g] = (uint32_t)i; }
    if (hi == g + 1) { right = 0x80000000u | (uint32_t)(g + 1); parent_leaf[g + 1] = (uint32_t)i; }
    else { right = (uint32_t)(g + 1); parent_int[g + 1] = (uint32_t)i; }
    child[2 * i] = left;
    child[2 * i + 1] = right;
    if (range) range[i] = make_uint2((uint32_t)lo, (uint32_t)hi);
}

__device__ __forceinline__ int bvh2_ref(uint32_t r) {
    return (r & 0x80000000u) ? ~(int)(r & 0x7fffffffu) : (int)r;
}

// Leaf boxes + refit. Each thread starts at a leaf; the second thread to
// arrive at a node computes its box from both children and continues upward.
// Exact boxes of internal nodes go to `nbox` (lo.xyz, hi.xyz as 2 float4);
// the child slots of each BVH2 node end up holding the children's boxes
// widened by widen_lo / widen_hi (traverse.cuh).
__global__ void k_refit(const float4* __restrict__ vpos, const uint4* __restrict__ tri_idx,
                        const uint32_t* __restrict__ order, const uint32_t* __restrict__ child,
                        const uint32_t* __restrict__ parent_int, const uint32_t* __restrict__ parent_leaf,
                        uint32_t n, unsigned int* __restrict__ flags, float4* __restrict__ nbox,
                        float4* __restrict__ nodes, float4* __restrict__ tri_wt, uint32_t prim_base = 0) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t prim = order[k];
    const uint4 ti = tri_idx[prim];
    const float4 a = vpos[ti.x], b = vpos[ti.y], c = vpos[ti.z];
    tri_wt[3 * (size_t)k + 0] = make_float4(a.x, a.y, a.z, __uint_as_float(prim_base + prim));
    tri_wt[3 * (size_t)k + 1] = make_float4(b.x, b.y, b.z, 0.0f);
    tri_wt[3 * (size_t)k + 2] = make_float4(c.x, c.y, c.z, 0.0f);
    float lo[3] = {fminf(fminf(a.x, b.x), c.x), fminf(fminf(a.y, b.y), c.y), fminf(fminf(a.z, b.z), c.z)};
    float hi[3] = {fmaxf(fmaxf(a.x, b.x), c.x), fmaxf(fmaxf(a.y, b.y), c.y), fmaxf(fmaxf(a.z, b.z), c.z)};
    if (n == 1) {
        // single triangle: one node whose two children are the same leaf.
        const float wl[3] = {widen_lo(lo[0]), widen_lo(lo[1]), widen_lo(lo[2])};
        const float wh[3] = {widen_hi(hi[0]), widen_hi(hi[1]), widen_hi(hi[2])};
        nodes[0] = make_float4(wl[0], wh[0], wl[1], wh[1]);
        nodes[1] = make_float4(wl[0], wh[0], wl[1], wh[1]);
        nodes[2] = make_float4(wl[2], wh[2], wl[2], wh[2]);
        nodes[3] = make_float4(__int_as_float(~0), __int_as_float(~0), 0.0f, 0.0f);
        nbox[0] = make_float4(lo[0], lo[1], lo[2], 0.0f);
        nbox[1] = make_float4(hi[0], hi[1], hi[2], 0.0f);
        return;
    }
    uint32_t cur = 0x80000000u | k;
    uint32_t p = parent_leaf[k];
    for (uint32_t steps = 0; steps < n; ++steps) {
        if (p >= n - 1) return;  // malformed parent link: stop (node left unset)
        const bool is_left = child[2 * p] == cur;
        float4* np = nodes + 4 * (size_t)p;
        if (is_left) {
            np[0] = make_float4(lo[0], hi[0], lo[1], hi[1]);
            reinterpret_cast<float2*>(np + 2)[0] = make_float2(lo[2], hi[2]);
        } else {
            np[1] = make_float4(lo[0], hi[0], lo[1], hi[1]);
            reinterpret_cast<float2*>(np + 2)[1] = make_float2(lo[2], hi[2]);
        }
        __threadfence();
        if (atomicAdd(flags + p, 1u) == 0u) return;
        __threadfence();
        const float4 s0 = __ldcg(np + 0), s1 = __ldcg(np + 1), s2 = __ldcg(np + 2);
        lo[0] = fminf(s0.x, s1.x); hi[0] = fmaxf(s0.y, s1.y);
        lo[1] = fminf(s0.z, s1.z); hi[1] = fmaxf(s0.w, s1.w);
        lo[2] = fminf(s2.x, s2.z); hi[2] = fmaxf(s2.y, s2.w);
        // the union above used the exact child boxes; the traversal reads
        // them widened (see slab_fma)
        np[0] = make_float4(widen_lo(s0.x), widen_hi(s0.y), widen_lo(s0.z), widen_hi(s0.w));
        np[1] = make_float4(widen_lo(s1.x), widen_hi(s1.y), widen_lo(s1.z), widen_hi(s1.w));
        np[2] = make_float4(widen_lo(s2.x), widen_hi(s2.y), widen_lo(s2.z), widen_hi(s2.w));
        np[3] = make_float4(__int_as_float(bvh2_ref(child[2 * p])), __int_as_float(bvh2_ref(child[2 * p + 1])),
                            0.0f, 0.0f);
        nbox[2 * (size_t)p + 0] = make_float4(lo[0], lo[1], lo[2], 0.0f);
        nbox[2 * (size_t)p + 1] = make_float4(hi[0], hi[1], hi[2], 0.0f);
        if (p == 0) return;
        cur = p;
        p = parent_int[p];
    }
}

// Depth of every leaf (ancestors + 1), reduced with atomicMax.
__global__ void k_depth(const uint32_t* __restrict__ parent_int, const uint32_t* __restrict__ parent_leaf,
                        uint32_t n, unsigned int* __restrict__ depth) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || n < 2) return;
    uint32_t d = 1;
    uint32_t p = parent_leaf[k];
    while (p != 0 && p < n - 1 && d < n) {
        p = parent_int[p];
        ++d;
    }
    atomicMax(depth, d + 1);
}

inline uint32_t blocks_for(uint64_t n, uint32_t b) { return (uint32_t)((n + b - 1) / b); }

// A wide BVH of `depth` levels must fit its traversal stack: BVH8 pushes
// one node group per level, BVH4 up to three node indices per level.
solrt_status check_wide_depth(uint32_t width, uint32_t depth) {
    if (width == 8 && depth > SOLRT_BVH8_STACK) {
        set_error("BVH8 depth %u exceeds the traversal stack (%d)", depth, SOLRT_BVH8_STACK);
        return SOLRT_ERR_CAPACITY;
    }
    if (width == 4 && 3u * depth + 1u > SOLRT_BVH2_STACK) {
        set_error("BVH4 depth %u exceeds the traversal stack (%d)", depth, SOLRT_BVH2_STACK);
        return SOLRT_ERR_CAPACITY;
    }
    return SOLRT_OK;
}

// BVH2-q16 (SOLRT_BVH2_Q16): the BVH2 with every child box stored as 16-bit
// planes of one grid per scene, a 32-byte node (one 256-bit load) instead of
// 64 bytes. Layout: a 32-byte header (grid origin G.xyz, cell c.x | c.y,
// c.z, ok flag, 0) followed by node i at byte 32 (i + 1):
//   (ref0, ref1, c0.x, c0.y, c0.z, c1.x, c1.y, c1.z)
// where each axis word packs the low plane in bits 0-15 and the high plane
// in bits 16-31; plane q of axis a lies at G.a + q c.a.
//
// Per axis the cell is the smallest power of two with extent / c <= 60000
// and c >= 2^-20 max|coordinate| (and 2^-60 <= c <= 2^23); G = floor(lo / c) c
// - 4 c. Planes are quantised outward from the (already widened) FP32 child
// boxes with two extra cells: the traversal's t = fma(2^23 + q, c / d,
// (G - o) / d - 2^23 c / d) differs from the exact plane distance by at most
// half a cell plus 3 * 2^-24 (|o| + |G|) / |d| plus 2^-24 |t|; the margin covers
// the first two for ray origins within twice the scene's coordinate range,
// and the relative 2^-16 widening of the far distance covers the rest (and
// the case of farther origins, where |t| ~ |o| / |d|).
__global__ void k_q16_grid(const float4* __restrict__ nbox, float4* __restrict__ header) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const float4 blo = nbox[0], bhi = nbox[1];
    const float lo[3] = {blo.x, blo.y, blo.z}, hi[3] = {bhi.x, bhi.y, bhi.z};
    float g[3], c[3];
    uint32_t ok = 1u;
    for (int a = 0; a < 3; ++a) {
        if (!isfinite(lo[a]) || !isfinite(hi[a]) || lo[a] > hi[a]) {
            ok = 0u;
            g[a] = 0.0f;
            c[a] = 1.0f;
            continue;
        }
        const double ext = (double)hi[a] - (double)lo[a];
        const double m = fmax(fabs((double)lo[a]), fabs((double)hi[a]));
        const double need = fmax(fmax(ext / 60000.0, m * 0x1p-20), 0x1p-60);
        int e = ilogb(need);
        if (ldexp(1.0, e) < need) ++e;
        if (e > 23) ok = 0u;
        const double cd = ldexp(1.0, e);
        c[a] = (float)cd;
        g[a] = (float)(floor((double)lo[a] / cd) * cd - 4.0 * cd);
    }
    header[0] = make_float4(g[0], g[1], g[2], c[0]);
    header[1] = make_float4(c[1], c[2], __uint_as_float(ok), 0.0f);
}

// Grid planes of one child axis: the low plane at least two cells below
// `lo`, the high plane two cells above `hi` (differences rounded outward,
// division by the power-of-two cell exact).
__device__ __forceinline__ uint32_t q16_pair(float lo, float hi, float g, float c) {
    const double dc = (double)c;
    const double ql = floor(__dsub_rd((double)lo, (double)g) / dc) - 2.0;
    const double qh = ceil(__dsub_ru((double)hi, (double)g) / dc) + 2.0;
    const uint32_t a = (uint32_t)fmin(fmax(ql, 0.0), 65535.0), b = (uint32_t)fmin(fmax(qh, 0.0), 65535.0);
    return a | (b << 16);
}

__global__ void k_q16_nodes(const float4* __restrict__ nodes, uint32_t ni, float4* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ni) return;
    const float4 h0 = out[0], h1 = out[1];
    const float g[3] = {h0.x, h0.y, h0.z}, c[3] = {h0.w, h1.x, h1.y};
    const float4 n0 = nodes[4 * (size_t)i], n1 = nodes[4 * (size_t)i + 1], n2 = nodes[4 * (size_t)i + 2],
                 n3 = nodes[4 * (size_t)i + 3];
    uint4* o = reinterpret_cast<uint4*>(out + 2 + 2 * (size_t)i);
    o[0] = make_uint4(__float_as_uint(n3.x), __float_as_uint(n3.y), q16_pair(n0.x, n0.y, g[0], c[0]),
                      q16_pair(n0.z, n0.w, g[1], c[1]));
    o[1] = make_uint4(q16_pair(n2.x, n2.y, g[2], c[2]), q16_pair(n1.x, n1.y, g[0], c[0]),
                      q16_pair(n1.z, n1.w, g[1], c[1]), q16_pair(n2.z, n2.w, g[2], c[2]));
}

// Replaces the 64-byte BVH2 nodes in `nodes` by the 32-byte BVH2-q16 nodes
// (header + ni nodes); `nbox` holds the exact internal-node boxes (root
// first). Fails when a coordinate is not finite or the scene is too large
// for the grid (synchronises to read the grid's flag).
solrt_status quantize_bvh2(Context& ctx, DeviceBuffer& nodes, const float4* nbox, uint32_t ni) {
    cudaStream_t st = ctx.stream;
    DeviceBuffer q;
    SOLRT_TRY(q.alloc(32ull * ((size_t)ni + 1)));
    k_q16_grid<<<1, 32, 0, st>>>(nbox, q.as<float4>());
    k_q16_nodes<<<blocks_for(ni, 256), 256, 0, st>>>(nodes.as<float4>(), ni, q.as<float4>());
    ctx.launches += 2;
    SOLRT_CUDA(cudaGetLastError());
    uint32_t ok = 0;
    SOLRT_CUDA(cudaMemcpyAsync(&ok, (const char*)q.ptr + 24, sizeof(ok), cudaMemcpyDeviceToHost, st));
    SOLRT_CUDA(cudaStreamSynchronize(st));
    if (ok != 1u) {
        set_error("BVH2_Q16: scene bounds are not finite or too large for a 16-bit grid (use SOLRT_BVH2)");
        return SOLRT_ERR_INVALID;
    }
    nodes.adopt(q);
    return SOLRT_OK;
}

}  // namespace

void launch_scan_exclusive(uint32_t* data, uint32_t len, cudaStream_t stream) {
    k_scan_exclusive<<<1, 1024, 0, stream>>>(data, len);
}

// Tile sums needed by scan_exclusive_tiled for `len` counts.
static uint32_t scan_tiles(uint32_t len) { return blocks_for(len, kScanTile); }

// Exclusive scan of `len` counts; `sums` holds scan_tiles(len) entries.
static void scan_exclusive_tiled(uint32_t* data, uint32_t len, uint32_t* sums, cudaStream_t stream) {
    const uint32_t tiles = scan_tiles(len);
    if (tiles <= 1) {
        k_scan_exclusive<<<1, 1024, 0, stream>>>(data, len);
        return;
    }
    k_scan_reduce<<<tiles, 1024, 0, stream>>>(data, len, sums);
    k_scan_exclusive<<<1, 1024, 0, stream>>>(sums, tiles);
    k_scan_apply<<<tiles, 1024, 0, stream>>>(data, len, sums);
}

// ---------------------------------------------------------------------------
// Two-level scenes (SOLRT_BVH2_TWO_LEVEL)
// ---------------------------------------------------------------------------

// Moves the references of `ni` BVH2 nodes built alone into the concatenated
// arrays: internal nodes by `node_off`, leaves by `tri_off`.
__global__ void k_offset_refs(float4* __restrict__ nodes, uint32_t ni, uint32_t node_off, uint32_t tri_off) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ni) return;
    float4 r = nodes[4 * (size_t)i + 3];
    int a = __float_as_int(r.x), b = __float_as_int(r.y);
    a = a >= 0 ? a + (int)node_off : ~((~a) + (int)tri_off);
    b = b >= 0 ? b + (int)node_off : ~((~b) + (int)tri_off);
    r.x = __int_as_float(a);
    r.y = __int_as_float(b);
    nodes[4 * (size_t)i + 3] = r;
}

// One binary LBVH over triangles tri_idx[0, n) of positions vpos: the
// 64-byte BVH2 nodes, the triangles in leaf order (prim = prim_base + index
// into tri_idx), and the topology and exact boxes the wide collapse and the
// refit reuse. Synchronises (reads the depth back).
struct Lbvh {
    uint32_t n = 0, ni = 0, depth = 0;
    DeviceBuffer nodes, tri_wt, child, par_int, par_leaf, range, nbox, order;
};

static solrt_status lbvh_build(Context& ctx, const float4* vpos, const uint4* tri_idx, uint32_t n, uint32_t prim_base,
                               Lbvh& L) {
    cudaStream_t st = ctx.stream;
    L.n = n;
    L.ni = n > 1 ? n - 1 : 1;  // internal nodes (one for a single triangle)
    const uint32_t ni = L.ni;
    DeviceBuffer cen, cb, keys[2], vals[2], hist, flags, depth;
    SOLRT_TRY(cen.alloc(sizeof(float4) * (size_t)n));
    SOLRT_TRY(cb.alloc(6 * sizeof(unsigned int)));
    for (int i = 0; i < 2; ++i) {
        SOLRT_TRY(keys[i].alloc(sizeof(uint32_t) * (size_t)n));
        SOLRT_TRY(vals[i].alloc(sizeof(uint32_t) * (size_t)n));
    }
    const uint32_t nblocks = blocks_for(n, kSortTile);
    SOLRT_TRY(hist.alloc(sizeof(uint32_t) * 256 * (size_t)nblocks));
    DeviceBuffer scan_sums;
    SOLRT_TRY(scan_sums.alloc(sizeof(uint32_t) * scan_tiles(256 * nblocks)));
    SOLRT_TRY(L.child.alloc(sizeof(uint32_t) * 2 * (size_t)ni));
    SOLRT_TRY(L.par_int.alloc(sizeof(uint32_t) * (size_t)ni));
    SOLRT_TRY(L.par_leaf.alloc(sizeof(uint32_t) * (size_t)n));
    SOLRT_TRY(flags.alloc(sizeof(unsigned int) * (size_t)ni));
    SOLRT_TRY(L.nbox.alloc(2 * sizeof(float4) * (size_t)ni));
    SOLRT_TRY(depth.alloc(sizeof(unsigned int)));
    SOLRT_TRY(L.range.alloc(sizeof(uint2) * (size_t)ni));
    SOLRT_TRY(L.nodes.alloc(4 * sizeof(float4) * (size_t)ni));
    SOLRT_TRY(L.tri_wt.alloc(3 * sizeof(float4) * (size_t)n));

    const unsigned int cb_init[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
    SOLRT_CUDA(cudaMemcpyAsync(cb.ptr, cb_init, sizeof(cb_init), cudaMemcpyHostToDevice, st));
    SOLRT_CUDA(cudaMemsetAsync(flags.ptr, 0, flags.bytes, st));
    SOLRT_CUDA(cudaMemsetAsync(depth.ptr, 0, depth.bytes, st));
    SOLRT_CUDA(cudaMemsetAsync(L.par_int.ptr, 0xff, L.par_int.bytes, st));

    k_centroids<<<blocks_for(n, 256), 256, 0, st>>>(vpos, tri_idx, n, cen.as<float4>(), cb.as<unsigned int>());
    k_morton<<<blocks_for(n, 256), 256, 0, st>>>(cen.as<float4>(), cb.as<unsigned int>(), n, keys[0].as<uint32_t>(),
                                                 vals[0].as<uint32_t>());
    int cur = 0;
    for (int shift = 0; shift < 30; shift += 8) {
        k_radix_hist<<<nblocks, kSortThreads, 0, st>>>(keys[cur].as<uint32_t>(), n, shift, nblocks,
                                                       hist.as<uint32_t>());
        scan_exclusive_tiled(hist.as<uint32_t>(), 256 * nblocks, scan_sums.as<uint32_t>(), st);
        k_radix_scatter<<<nblocks, kSortThreads, 0, st>>>(keys[cur].as<uint32_t>(), vals[cur].as<uint32_t>(),
                                                          keys[cur ^ 1].as<uint32_t>(), vals[cur ^ 1].as<uint32_t>(),
                                                          hist.as<uint32_t>(), n, shift, nblocks);
        cur ^= 1;
        ctx.launches += 3;
    }
    if (n > 1) {
        k_karras<<<blocks_for(n - 1, 256), 256, 0, st>>>(keys[cur].as<uint32_t>(), n, L.child.as<uint32_t>(),
                                                         L.par_int.as<uint32_t>(), L.par_leaf.as<uint32_t>(),
                                                         L.range.as<uint2>());
        ++ctx.launches;
    }
    k_refit<<<blocks_for(n, 256), 256, 0, st>>>(vpos, tri_idx, vals[cur].as<uint32_t>(), L.child.as<uint32_t>(),
                                                L.par_int.as<uint32_t>(), L.par_leaf.as<uint32_t>(), n,
                                                flags.as<unsigned int>(), L.nbox.as<float4>(), L.nodes.as<float4>(),
                                                L.tri_wt.as<float4>(), prim_base);
    k_depth<<<blocks_for(n, 256), 256, 0, st>>>(L.par_int.as<uint32_t>(), L.par_leaf.as<uint32_t>(), n,
                                                depth.as<unsigned int>());
    ctx.launches += 5;
    SOLRT_CUDA(cudaGetLastError());
    L.order.adopt(vals[cur]);
    unsigned int dh = 0;
    SOLRT_CUDA(cudaMemcpyAsync(&dh, depth.ptr, sizeof(dh), cudaMemcpyDeviceToHost, st));
    SOLRT_CUDA(cudaStreamSynchronize(st));
    L.depth = n > 1 ? dh : 1;
    return SOLRT_OK;
}

// TLAS of a two-level scene, built on the host from the staged instances:
// each non-empty section's object-space root box is transformed (8 corners,
// FP64), rounded outward to float and widened like every BVH2 child box,
// then the instance boxes are split at the median centroid of their widest
// axis. Node 0 is the root; leaves are ~section. Uploads the TLAS nodes and
// the instance table (inverse-transform rows = transform_it transposed, and
// the section's BLAS root).
static float host_int_as_float(int v) {
    float f;
    std::memcpy(&f, &v, sizeof(f));
    return f;
}

static solrt_status build_tlas(Context& ctx, Scene& sc) {
    struct IBox {
        float lo[3], hi[3], c[3];
        int32_t sec;
    };
    const uint32_t S = sc.section_count;
    std::vector<IBox> items;
    for (uint32_t s = 0; s < S; ++s) {
        if (sc.blas_root.size() <= s || sc.blas_root[s] < 0) continue;
        const float* T = sc.inst_host[s].transform;  // column-major
        double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int k = 0; k < 8; ++k) {
            const double v[3] = {sc.blas_box[6 * s + ((k & 1) ? 3 : 0)], sc.blas_box[6 * s + 1 + ((k & 2) ? 3 : 0)],
                                 sc.blas_box[6 * s + 2 + ((k & 4) ? 3 : 0)]};
            for (int r = 0; r < 3; ++r) {
                const double w = (double)T[r] * v[0] + (double)T[4 + r] * v[1] + (double)T[8 + r] * v[2] +
                                 (double)T[12 + r];
                lo[r] = std::min(lo[r], w);
                hi[r] = std::max(hi[r], w);
            }
        }
        IBox b;
        for (int r = 0; r < 3; ++r) {
            if (!std::isfinite(lo[r]) || !std::isfinite(hi[r]) || std::fabs(lo[r]) > 1e37 || std::fabs(hi[r]) > 1e37) {
                set_error("instance %u: transformed bounds are not finite", s);
                return SOLRT_ERR_INVALID;
            }
            float fl = (float)lo[r], fh = (float)hi[r];
            if ((double)fl > lo[r]) fl = std::nextafter(fl, -INFINITY);
            if ((double)fh < hi[r]) fh = std::nextafter(fh, INFINITY);
            b.lo[r] = widen_lo(fl);
            b.hi[r] = widen_hi(fh);
            b.c[r] = 0.5f * (b.lo[r] + b.hi[r]);
        }
        b.sec = (int32_t)s;
        items.push_back(b);
    }
    std::vector<float4> nodes;
    uint32_t depth = 0;
    auto box_of = [&](size_t a, size_t e, float* lo, float* hi) {
        for (int r = 0; r < 3; ++r) {
            lo[r] = INFINITY;
            hi[r] = -INFINITY;
        }
        for (size_t i = a; i < e; ++i)
            for (int r = 0; r < 3; ++r) {
                lo[r] = std::min(lo[r], items[i].lo[r]);
                hi[r] = std::max(hi[r], items[i].hi[r]);
            }
    };
    auto put_node = [&](size_t id, const float* l0, const float* h0, const float* l1, const float* h1, int r0,
                        int r1) {
        nodes[4 * id + 0] = make_float4(l0[0], h0[0], l0[1], h0[1]);
        nodes[4 * id + 1] = make_float4(l1[0], h1[0], l1[1], h1[1]);
        nodes[4 * id + 2] = make_float4(l0[2], h0[2], l1[2], h1[2]);
        nodes[4 * id + 3] = make_float4(host_int_as_float(r0), host_int_as_float(r1), 0.0f, 0.0f);
    };
    // explicit stack of (first, end, node slot, depth); children are built
    // after their parent so node 0 is the root
    struct Task {
        size_t a, e, id;
        uint32_t d;
    };
    if (items.size() == 1) {  // one instance: both children are that leaf
        nodes.resize(4);
        put_node(0, items[0].lo, items[0].hi, items[0].lo, items[0].hi, ~items[0].sec, ~items[0].sec);
        depth = 1;
    } else if (items.size() > 1) {
        nodes.resize(4);
        std::vector<Task> todo{{0, items.size(), 0, 1}};
        while (!todo.empty()) {
            const Task t = todo.back();
            todo.pop_back();
            depth = std::max(depth, t.d);
            float clo[3], chi[3];
            for (int r = 0; r < 3; ++r) {
                clo[r] = INFINITY;
                chi[r] = -INFINITY;
            }
            for (size_t i = t.a; i < t.e; ++i)
                for (int r = 0; r < 3; ++r) {
                    clo[r] = std::min(clo[r], items[i].c[r]);
                    chi[r] = std::max(chi[r], items[i].c[r]);
                }
            int axis = 0;
            for (int r = 1; r < 3; ++r)
                if (chi[r] - clo[r] > chi[axis] - clo[axis]) axis = r;
            std::sort(items.begin() + (long)t.a, items.begin() + (long)t.e, [&](const IBox& x, const IBox& y) {
                return x.c[axis] != y.c[axis] ? x.c[axis] < y.c[axis] : x.sec < y.sec;
            });
            const size_t mid = t.a + (t.e - t.a) / 2;
            float l0[3], h0[3], l1[3], h1[3];
            box_of(t.a, mid, l0, h0);
            box_of(mid, t.e, l1, h1);
            int refs[2];
            const size_t ranges[2][2] = {{t.a, mid}, {mid, t.e}};
            for (int side = 0; side < 2; ++side) {
                const size_t a = ranges[side][0], e = ranges[side][1];
                if (e - a == 1) {
                    refs[side] = ~items[a].sec;
                } else {
                    const size_t id = nodes.size() / 4;
                    nodes.resize(nodes.size() + 4);
                    refs[side] = (int)id;
                    todo.push_back({a, e, id, t.d + 1});
                }
            }
            put_node(t.id, l0, h0, l1, h1, refs[0], refs[1]);
        }
    }
    sc.tlas_count = (uint32_t)(nodes.size() / 4);
    sc.tlas_depth = depth;
    if (sc.blas_depth + sc.tlas_depth + 2 > SOLRT_BVH2_STACK) {
        set_error("two-level depth %u + %u exceeds the traversal stack (%d)", sc.tlas_depth, sc.blas_depth,
                  SOLRT_BVH2_STACK);
        return SOLRT_ERR_CAPACITY;
    }
    std::vector<float4> table(4 * (size_t)S);
    for (uint32_t s = 0; s < S; ++s) {
        const float* Ti = sc.inst_host[s].transform_it;  // column-major; row r of its transpose = Ti[4r..4r+3]
        for (int r = 0; r < 3; ++r) table[4 * s + r] = make_float4(Ti[4 * r], Ti[4 * r + 1], Ti[4 * r + 2], Ti[4 * r + 3]);
        table[4 * s + 3] = make_float4(host_int_as_float(sc.blas_root.size() > s ? sc.blas_root[s] : -1), 0.0f,
                                       0.0f, 0.0f);
    }
    cudaStream_t st = ctx.stream;
    if (sc.tlas_count) {
        SOLRT_TRY(sc.tlas.alloc(sizeof(float4) * nodes.size()));
        SOLRT_CUDA(cudaMemcpyAsync(sc.tlas.ptr, nodes.data(), sizeof(float4) * nodes.size(), cudaMemcpyHostToDevice, st));
    }
    if (S) {
        SOLRT_TRY(sc.inst_table.alloc(sizeof(float4) * table.size()));
        SOLRT_CUDA(cudaMemcpyAsync(sc.inst_table.ptr, table.data(), sizeof(float4) * table.size(),
                                   cudaMemcpyHostToDevice, st));
    }
    SOLRT_CUDA(cudaStreamSynchronize(st));  // the host arrays go out of scope
    return SOLRT_OK;
}

// The BLASes of a two-level scene: one LBVH per non-empty section over its
// object-space triangles, concatenated (nodes, then triangles in the
// sections' order), then the TLAS.
// A binary LBVH to restructure by treelets, with the geometry lbvh_build got.
struct TreeletInput {
    const float4* vpos;
    const uint4* tri_idx;
    uint32_t prim_base;
    Lbvh* L;
};
static solrt_status treelet_restructure(Context& ctx, const std::vector<TreeletInput>& in, int rounds);
constexpr int kTreeletRoundsTwoLevel = 3;

static solrt_status build_two_level(Context& ctx, Scene& sc) {
    cudaStream_t st = ctx.stream;
    const uint32_t S = sc.section_count;
    if (!sc.opos.ptr || sc.sec_tri_first.size() != S || sc.inst_host.size() != S) {
        set_error("a two-level BVH needs a scene created with SOLRT_BVH2_TWO_LEVEL (object-space geometry)");
        return SOLRT_ERR_INVALID;
    }
    uint64_t total = 0;
    for (uint32_t s = 0; s < S; ++s)
        if (sc.sec_tri_count[s]) total += sc.sec_tri_count[s] > 1 ? sc.sec_tri_count[s] - 1 : 1;
    SOLRT_TRY(sc.nodes.alloc(4 * sizeof(float4) * std::max<uint64_t>(total, 1)));
    SOLRT_TRY(sc.tri_wt.alloc(3 * sizeof(float4) * (size_t)sc.tri_count));
    sc.blas_box.assign(6 * (size_t)S, 0.0f);
    sc.blas_root.assign(S, -1);
    sc.blas_depth = 0;
    // every section's LBVH, then (SOLRT_BVH_SAH) all of them restructured
    // together, one k_treelet launch per round
    std::unique_ptr<Lbvh[]> Ls(new (std::nothrow) Lbvh[S]);
    if (!Ls) return SOLRT_ERR_OOM;
    std::vector<TreeletInput> tin;
    for (uint32_t s = 0; s < S; ++s) {
        const uint32_t cnt = sc.sec_tri_count[s], first = sc.sec_tri_first[s];
        if (cnt == 0) continue;
        SOLRT_TRY(lbvh_build(ctx, sc.opos.as<float4>(), sc.tri_idx.as<uint4>() + first, cnt, first, Ls[s]));
        tin.push_back(TreeletInput{sc.opos.as<float4>(), sc.tri_idx.as<uint4>() + first, first, &Ls[s]});
    }
    if (sc.desc.flags & SOLRT_BVH_SAH) SOLRT_TRY(treelet_restructure(ctx, tin, kTreeletRoundsTwoLevel));
    std::vector<float4> boxes(2 * (size_t)S);
    uint32_t node_off = 0;
    for (uint32_t s = 0; s < S; ++s) {
        const uint32_t cnt = sc.sec_tri_count[s], first = sc.sec_tri_first[s];
        if (cnt == 0) continue;
        const Lbvh& L = Ls[s];
        SOLRT_CUDA(cudaMemcpyAsync(sc.nodes.as<float4>() + 4 * (size_t)node_off, L.nodes.ptr,
                                   4 * sizeof(float4) * (size_t)L.ni, cudaMemcpyDeviceToDevice, st));
        SOLRT_CUDA(cudaMemcpyAsync(sc.tri_wt.as<float4>() + 3 * (size_t)first, L.tri_wt.ptr,
                                   3 * sizeof(float4) * (size_t)cnt, cudaMemcpyDeviceToDevice, st));
        k_offset_refs<<<blocks_for(L.ni, 256), 256, 0, st>>>(sc.nodes.as<float4>() + 4 * (size_t)node_off, L.ni,
                                                            node_off, first);
        ++ctx.launches;
        SOLRT_CUDA(cudaGetLastError());
        SOLRT_CUDA(cudaMemcpyAsync(boxes.data() + 2 * (size_t)s, L.nbox.ptr, 2 * sizeof(float4),
                                   cudaMemcpyDeviceToHost, st));
        sc.blas_root[s] = (int32_t)node_off;
        node_off += L.ni;
        sc.blas_depth = std::max(sc.blas_depth, L.depth);
    }
    SOLRT_CUDA(cudaStreamSynchronize(st));
    for (uint32_t s = 0; s < S; ++s) {
        if (sc.sec_tri_count[s] == 0) continue;
        const float4 lo = boxes[2 * (size_t)s], hi = boxes[2 * (size_t)s + 1];
        const float b[6] = {lo.x, lo.y, lo.z, hi.x, hi.y, hi.z};
        for (int i = 0; i < 6; ++i) sc.blas_box[6 * s + i] = b[i];
    }
    sc.info.node_count = node_off;
    sc.info.node_bytes = 64ull * node_off;
    SOLRT_TRY(build_tlas(ctx, sc));
    sc.info.depth = sc.blas_depth + sc.tlas_depth;
    return SOLRT_OK;
}

// The single-level kinds: one LBVH over the world-space triangles, then the
// wide collapse or the 16-bit quantisation when asked.
// ---------------------------------------------------------------------------
// Treelet restructuring of the LBVH toward the SAH (Karras and Aila, "Fast
// parallel construction of high-quality bounding volume hierarchies", HPG
// 2013), for the binary kinds with SOLRT_BVH_SAH. Bottom up, as the refit
// walks: the second thread to reach an internal node owns its subtree, and
// its warp processes the node's treelet, all 32 lanes together, one owned
// node after another (the top of the tree, where one node at a time is
// ready, is the latency of the whole pass). The treelet grows from the
// node's two children by replacing the internal treelet leaf of largest
// surface area with its two children until it has kTreeletLeaves leaves (or
// only triangles are left; lane q holds leaf q); a dynamic program over the
// subsets of those leaves, one subset size after another with a subset per
// lane, finds the binary tree of least SAH cost (node visit 1, triangle test
// kSahTri, per unit of surface area); when that is cheaper than the subtree
// as it is, the treelet's internal nodes are rewritten (the node itself
// stays the treelet's root, the expanded nodes are reused in expansion
// order). Leaves keep their positions in the leaf order, so the triangle
// stream is unchanged; only child and parent links, exact boxes and subtree
// costs change. Deterministic: a node's result depends only on its subtree,
// which is final when the node is processed, and ties go to the first
// candidate in a fixed order (the lowest leaf; the first partition in the
// submask order).
// ---------------------------------------------------------------------------

namespace {

constexpr int kTreeletLeaves = 7;
constexpr int kTreeletRounds = 3;
constexpr int kTreeletWarps = 4;  // warps per block of k_treelet
constexpr float kSahTri = 0.3f;

SOLRT_D float box_area(const float b[6]) {
    const float ex = fmaxf(b[3] - b[0], 0.0f), ey = fmaxf(b[4] - b[1], 0.0f), ez = fmaxf(b[5] - b[2], 0.0f);
    return 2.0f * ((ex * ey + ey * ez) + ez * ex);
}

// Exact box (lo.xyz, hi.xyz) of a child reference: a leaf's triangle from
// the leaf-ordered stream, an internal node's from `nbox` (written by other
// warps: read through L2).
SOLRT_D void ref_box(uint32_t ref, const float4* __restrict__ tri_wt, const float4* nbox, float b[6]) {
    if (ref & 0x80000000u) {
        const size_t k = ref & 0x7fffffffu;
        const float4 a = tri_wt[3 * k], c = tri_wt[3 * k + 1], d = tri_wt[3 * k + 2];
        b[0] = fminf(fminf(a.x, c.x), d.x); b[1] = fminf(fminf(a.y, c.y), d.y); b[2] = fminf(fminf(a.z, c.z), d.z);
        b[3] = fmaxf(fmaxf(a.x, c.x), d.x); b[4] = fmaxf(fmaxf(a.y, c.y), d.y); b[5] = fmaxf(fmaxf(a.z, c.z), d.z);
    } else {
        const float4 lo = __ldcg(nbox + 2 * (size_t)ref), hi = __ldcg(nbox + 2 * (size_t)ref + 1);
        b[0] = lo.x; b[1] = lo.y; b[2] = lo.z; b[3] = hi.x; b[4] = hi.y; b[5] = hi.z;
    }
}

// A warp's working set for one treelet.
struct TreeletSmem {
    float cs[1 << kTreeletLeaves];    // least SAH cost of each subset of treelet leaves
    float ar[1 << kTreeletLeaves];    // surface area of each subset's box
    uint8_t part[1 << kTreeletLeaves];  // its best first part (a subset holding the lowest leaf)
    float lb[kTreeletLeaves][6];      // leaf boxes
    uint32_t lref[kTreeletLeaves];    // leaf references
    uint32_t inner[kTreeletLeaves - 2];  // expanded internal nodes, in expansion order
};

SOLRT_D void subset_box(const TreeletSmem& s, uint32_t S, int nl, float b[6]) {
    b[0] = b[1] = b[2] = INFINITY;
    b[3] = b[4] = b[5] = -INFINITY;
    for (int q = 0; q < nl; ++q)
        if (S & (1u << q))
            for (int a = 0; a < 3; ++a) {
                b[a] = fminf(b[a], s.lb[q][a]);
                b[3 + a] = fmaxf(b[3 + a], s.lb[q][3 + a]);
            }
}

// The treelet of node p, by all 32 lanes of the calling warp.
SOLRT_D void treelet_warp(uint32_t p, TreeletSmem& s, const float4* __restrict__ tri_wt, uint32_t* child,
                          uint32_t* par_int, uint32_t* par_leaf, float4* nbox, float* cost) {
    const uint32_t lane = threadIdx.x & 31u;
    // lanes 0 and 1 start with the node's children; lane q holds leaf q
    uint32_t ref = 0xffffffffu;
    float b[6], area = -1.0f, kinit = 0.0f;
    if (lane < 2) {
        ref = __ldcg(child + 2 * (size_t)p + lane);
        ref_box(ref, tri_wt, nbox, b);
        area = box_area(b);
        kinit = (ref & 0x80000000u) ? kSahTri * area : __ldcg(cost + ref);
    }
    const float k0 = __shfl_sync(0xffffffffu, kinit, 0), k1 = __shfl_sync(0xffffffffu, kinit, 1);
    int nl = 2, nin = 0;
    uint32_t inner = 0;  // lane i holds the i-th expanded node
    while (nl < kTreeletLeaves) {
        // the internal leaf of largest area, the lowest index among equals
        float best = ((int)lane < nl && !(ref & 0x80000000u) && area >= 0.0f) ? area : -1.0f;
        uint32_t bi = lane;
#pragma unroll
        for (int off = 16; off; off >>= 1) {
            const float ob = __shfl_xor_sync(0xffffffffu, best, off);
            const uint32_t oi = __shfl_xor_sync(0xffffffffu, bi, off);
            if (ob > best || (ob == best && oi < bi)) {
                best = ob;
                bi = oi;
            }
        }
        if (best < 0.0f) break;  // only triangles left
        const uint32_t r = __shfl_sync(0xffffffffu, ref, bi);
        if ((int)lane == nin) inner = r;
        ++nin;
        if (lane == bi || (int)lane == nl) {
            ref = __ldcg(child + 2 * (size_t)r + (lane == bi ? 0u : 1u));
            ref_box(ref, tri_wt, nbox, b);
            area = box_area(b);
        }
        ++nl;
    }
    if ((int)lane < nl) {
        for (int a = 0; a < 6; ++a) s.lb[lane][a] = b[a];
        s.lref[lane] = ref;
        s.cs[1u << lane] = (ref & 0x80000000u) ? kSahTri * area : __ldcg(cost + ref);
        s.part[1u << lane] = 0;
    }
    if ((int)lane < nin) s.inner[lane] = inner;
    __syncwarp();
    const uint32_t full = (1u << nl) - 1u;
    for (uint32_t S = lane + 1u; S <= full; S += 32u) {
        float u[6];
        subset_box(s, S, nl, u);
        s.ar[S] = box_area(u);
    }
    __syncwarp();
    // cost of the subtree as it stands: its two children are final
    const float cur = s.ar[full] + (k0 + k1);
    bool rebuild = false;
    if (nl >= 3) {
        for (int sz = 2; sz <= nl; ++sz) {
            for (uint32_t S = lane + 1u; S <= full; S += 32u) {
                if (__popc(S) != sz) continue;
                const uint32_t low = S & (0u - S);
                float bestv = INFINITY;
                uint32_t bp = low;
                for (uint32_t P = (S - 1u) & S; P != 0u; P = (P - 1u) & S) {
                    if (!(P & low)) continue;
                    const float v = s.cs[P] + s.cs[S ^ P];
                    if (v < bestv) {
                        bestv = v;
                        bp = P;
                    }
                }
                s.cs[S] = s.ar[S] + bestv;
                s.part[S] = (uint8_t)bp;
            }
            __syncwarp();
        }
        rebuild = s.cs[full] < cur * (1.0f - 1e-5f);
    }
    if (lane == 0) {
        if (rebuild) {
            // rewrite the treelet top down: (subset, node) pairs
            uint32_t stS[kTreeletLeaves], stN[kTreeletLeaves];
            int sp = 0, used = 0;
            stS[sp] = full;
            stN[sp++] = p;
            while (sp > 0) {
                const uint32_t S = stS[--sp], node = stN[sp];
                float u[6];
                subset_box(s, S, nl, u);
                nbox[2 * (size_t)node] = make_float4(u[0], u[1], u[2], 0.0f);
                nbox[2 * (size_t)node + 1] = make_float4(u[3], u[4], u[5], 0.0f);
                cost[node] = s.cs[S];
                const uint32_t sides[2] = {s.part[S], S ^ s.part[S]};
#pragma unroll
                for (int side = 0; side < 2; ++side) {
                    const uint32_t T = sides[side];
                    uint32_t cref;
                    if ((T & (T - 1u)) == 0u) {
                        cref = s.lref[__ffs(T) - 1];
                        if (cref & 0x80000000u) par_leaf[cref & 0x7fffffffu] = node;
                        else par_int[cref] = node;
                    } else {
                        cref = s.inner[used++];
                        par_int[cref] = node;
                        stS[sp] = T;
                        stN[sp++] = cref;
                    }
                    child[2 * (size_t)node + side] = cref;
                }
            }
        } else {
            float u[6];
            subset_box(s, full, nl, u);
            nbox[2 * (size_t)p] = make_float4(u[0], u[1], u[2], 0.0f);
            nbox[2 * (size_t)p + 1] = make_float4(u[3], u[4], u[5], 0.0f);
            cost[p] = cur;
        }
    }
    __syncwarp();
}

// One binary LBVH of a k_treelet launch: its arrays, its triangle count
// (at least 3) and its first block (blocks [block0, block0 + its leaves /
// block size) of the launch are its own).
struct TreeletTree {
    const float4* tri_wt;
    uint32_t* child;
    uint32_t* par_int;
    uint32_t* par_leaf;
    float4* nbox;
    float* cost;
    unsigned int* flags;
    uint32_t n, block0;
};

// One round over each tree of `trees` (ascending block0, the first 0): one
// thread per leaf walks up; the lanes that own a node this step hand it to
// their warp in turn. Every lane stays in the loop until its warp is done,
// so the warp-wide steps see all 32 lanes.
__global__ void __launch_bounds__(32 * kTreeletWarps) k_treelet(const TreeletTree* __restrict__ trees,
                                                                uint32_t ntrees) {
    __shared__ TreeletSmem smem[kTreeletWarps];
    TreeletSmem& s = smem[threadIdx.x >> 5];
    uint32_t lo = 0, hi = ntrees - 1u;  // the last tree with block0 <= blockIdx.x
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1u) >> 1;
        if (trees[mid].block0 <= blockIdx.x) lo = mid;
        else hi = mid - 1u;
    }
    const TreeletTree T = trees[lo];
    const float4* tri_wt = T.tri_wt;
    uint32_t *child = T.child, *par_int = T.par_int, *par_leaf = T.par_leaf;
    float4* nbox = T.nbox;
    float* cost = T.cost;
    unsigned int* flags = T.flags;
    const uint32_t n = T.n;
    const uint32_t k = (blockIdx.x - T.block0) * blockDim.x + threadIdx.x;
    bool active = k < n;
    uint32_t p = active ? par_leaf[k] : 0u;
    for (uint32_t steps = 0; steps < n; ++steps) {
        bool own = false;
        if (active) {
            if (p >= n - 1) {
                active = false;  // malformed parent link
            } else {
                __threadfence();
                if (atomicAdd(flags + p, 1u) == 0u) active = false;  // the sibling subtree is not done yet
                else own = true;
            }
        }
        __threadfence();
        uint32_t m = __ballot_sync(0xffffffffu, own);
        if (m == 0u) break;  // every lane has stopped
        while (m) {
            const int l = __ffs(m) - 1;
            m &= m - 1u;
            treelet_warp(__shfl_sync(0xffffffffu, p, l), s, tri_wt, child, par_int, par_leaf, nbox, cost);
        }
        __threadfence();
        if (own) {
            if (p == 0) active = false;
            else p = __ldcg(par_int + p);
        }
    }
}

}  // namespace

// Restructures the binary LBVHs of `in` in place (rounds of k_treelet, each
// one launch over all of them), then writes each one's nodes again (k_refit)
// and its depth. Synchronises.
static solrt_status treelet_restructure(Context& ctx, const std::vector<TreeletInput>& in, int rounds) {
    cudaStream_t st = ctx.stream;
    std::vector<TreeletTree> trees;
    std::vector<size_t> off;  // each tree's first entry in flags / cost
    size_t total = 0;
    uint32_t blocks = 0;
    for (const TreeletInput& t : in) {
        if (t.L->n < 3) continue;
        trees.push_back(TreeletTree{t.L->tri_wt.as<float4>(), t.L->child.as<uint32_t>(), t.L->par_int.as<uint32_t>(),
                                    t.L->par_leaf.as<uint32_t>(), t.L->nbox.as<float4>(), nullptr, nullptr, t.L->n,
                                    blocks});
        off.push_back(total);
        total += t.L->ni;
        blocks += blocks_for(t.L->n, 32 * kTreeletWarps);
    }
    if (trees.empty()) return SOLRT_OK;
    const uint32_t nt = (uint32_t)trees.size();
    DeviceBuffer flags, cost, depth, table;
    SOLRT_TRY(flags.alloc(sizeof(unsigned int) * total));
    SOLRT_TRY(cost.alloc(sizeof(float) * total));
    SOLRT_TRY(depth.alloc(sizeof(unsigned int) * (size_t)nt));
    SOLRT_TRY(table.alloc(sizeof(TreeletTree) * (size_t)nt));
    for (uint32_t i = 0; i < nt; ++i) {
        trees[i].flags = flags.as<unsigned int>() + off[i];
        trees[i].cost = cost.as<float>() + off[i];
    }
    SOLRT_CUDA(cudaMemcpyAsync(table.ptr, trees.data(), sizeof(TreeletTree) * (size_t)nt, cudaMemcpyHostToDevice, st));
    for (int r = 0; r < rounds; ++r) {
        SOLRT_CUDA(cudaMemsetAsync(flags.ptr, 0, flags.bytes, st));
        k_treelet<<<blocks, 32 * kTreeletWarps, 0, st>>>(table.as<TreeletTree>(), nt);
        ++ctx.launches;
    }
    SOLRT_CUDA(cudaMemsetAsync(flags.ptr, 0, flags.bytes, st));
    SOLRT_CUDA(cudaMemsetAsync(depth.ptr, 0, depth.bytes, st));
    uint32_t i = 0;
    for (const TreeletInput& t : in) {
        Lbvh& L = *t.L;
        if (L.n < 3) continue;
        k_refit<<<blocks_for(L.n, 256), 256, 0, st>>>(t.vpos, t.tri_idx, L.order.as<uint32_t>(), L.child.as<uint32_t>(),
                                                      L.par_int.as<uint32_t>(), L.par_leaf.as<uint32_t>(), L.n,
                                                      flags.as<unsigned int>() + off[i], L.nbox.as<float4>(),
                                                      L.nodes.as<float4>(), L.tri_wt.as<float4>(), t.prim_base);
        k_depth<<<blocks_for(L.n, 256), 256, 0, st>>>(L.par_int.as<uint32_t>(), L.par_leaf.as<uint32_t>(), L.n,
                                                      depth.as<unsigned int>() + i);
        ctx.launches += 2;
        ++i;
    }
    SOLRT_CUDA(cudaGetLastError());
    std::vector<unsigned int> dh(nt);
    SOLRT_CUDA(cudaMemcpyAsync(dh.data(), depth.ptr, sizeof(unsigned int) * (size_t)nt, cudaMemcpyDeviceToHost, st));
    SOLRT_CUDA(cudaStreamSynchronize(st));
    i = 0;
    for (const TreeletInput& t : in)
        if (t.L->n >= 3) t.L->depth = dh[i++];
    return SOLRT_OK;
}

static solrt_status build_single_level(Context& ctx, Scene& sc, const solrt_bvh_desc& desc) {
    const uint32_t n = sc.tri_count;
    Lbvh L;
    SOLRT_TRY(lbvh_build(ctx, sc.vpos.as<float4>(), sc.tri_idx.as<uint4>(), n, 0u, L));
    // Treelets for the binary kinds, and for the wide kinds when every leaf
    // slot holds one triangle: their collapse then reads a node's leaf range
    // only as "more than one triangle", which restructuring keeps true (a
    // restructured node's leaves need not be contiguous any more).
    const bool wide = desc.kind == SOLRT_BVH8_Q8 || desc.kind == SOLRT_BVH4_Q8 || desc.kind == SOLRT_BVH8_F32;
    if ((desc.flags & SOLRT_BVH_SAH) && (!wide || desc.leaf_max <= 1u))
        SOLRT_TRY(treelet_restructure(ctx, {TreeletInput{sc.vpos.as<float4>(), sc.tri_idx.as<uint4>(), 0u, &L}},
                                      kTreeletRounds));
    const uint32_t ni = L.ni;
    if (desc.kind == SOLRT_BVH8_Q8 || desc.kind == SOLRT_BVH4_Q8 || desc.kind == SOLRT_BVH8_F32) {
        const uint32_t width = desc.kind == SOLRT_BVH4_Q8 ? 4u : 8u;
        const bool f32 = desc.kind == SOLRT_BVH8_F32;
        Bvh8BuildInput in;
        in.n = n;
        in.child = L.child.as<uint32_t>();
        in.nbox = L.nbox.as<float4>();
        in.range = L.range.as<uint2>();
        in.tri_wt_leaf = L.tri_wt.as<float4>();
        in.leaf_max = desc.leaf_max == 0 ? 1u : std::min(3u, desc.leaf_max);
        in.par_int = L.par_int.as<uint32_t>();
        in.par_leaf = L.par_leaf.as<uint32_t>();
        in.sah = (desc.flags & SOLRT_BVH_SAH) != 0;
        DeviceBuffer tri8;
        uint32_t node_count = 0, depth8 = 0;
        SOLRT_TRY(build_wide(ctx, in, width, f32, sc.nodes, tri8, &node_count, &depth8));
        sc.tri_wt.adopt(tri8);
        sc.info.node_count = node_count;
        sc.info.depth = depth8;
        sc.info.node_bytes = (uint64_t)node_count * (width == 4 ? 64u : (f32 ? 224u : 80u));
        SOLRT_TRY(check_wide_depth(width, depth8));
    } else {
        sc.nodes.adopt(L.nodes);
        sc.tri_wt.adopt(L.tri_wt);
        sc.info.node_count = ni;
        sc.info.node_bytes = (uint64_t)ni * 64u;
        if (desc.kind == SOLRT_BVH2_Q16) {
            SOLRT_TRY(quantize_bvh2(ctx, sc.nodes, L.nbox.as<float4>(), ni));
            sc.info.node_bytes = 32ull * ((uint64_t)ni + 1);
        }
        sc.info.depth = L.depth;
    }
    if (sc.dynamic) {  // the topology stays for solrt_scene_regenerate(REFIT)
        sc.topo_order.adopt(L.order);
        sc.topo_child.adopt(L.child);
        sc.topo_par_int.adopt(L.par_int);
        sc.topo_par_leaf.adopt(L.par_leaf);
        sc.topo_range.adopt(L.range);
    }
    return SOLRT_OK;
}

// Builds the LBVH of `sc` (and the wide collapse or the 16-bit quantisation
// when asked). Scratch is allocated for the duration of the build.
// Synchronises.
solrt_status build_bvh(Context& ctx, Scene& sc, const solrt_bvh_desc& desc) {
    const uint32_t n = sc.tri_count;
    cudaStream_t st = ctx.stream;
    sc.info = solrt_bvh_info{};
    sc.info.kind = desc.kind;
    sc.info.tri_count = n;
    sc.nodes.release();
    sc.tri_wt.release();
    sc.desc = desc;
    if (n == 0) return SOLRT_OK;
    cudaGetLastError();  // launch errors below must be this call's own

    SOLRT_CUDA(cudaEventRecord(ctx.ev0, st));
    if (desc.kind == SOLRT_BVH2_TWO_LEVEL) SOLRT_TRY(build_two_level(ctx, sc));
    else SOLRT_TRY(build_single_level(ctx, sc, desc));
    sc.info.tri_bytes = sc.tri_wt.bytes;
    sc.info.shade_bytes = sc.opos.bytes + sc.vnc.bytes + sc.tri_idx.bytes + sc.materials.bytes +
                          sc.instances.bytes + sc.sec_mat.bytes;
    SOLRT_CUDA(cudaEventRecord(ctx.ev1, st));
    SOLRT_CUDA(cudaEventSynchronize(ctx.ev1));
    float ms = 0.0f;
    SOLRT_CUDA(cudaEventElapsedTime(&ms, ctx.ev0, ctx.ev1));
    sc.info.build_ms = ms;
    if ((sc.info.kind == SOLRT_BVH2 || sc.info.kind == SOLRT_BVH2_Q16) && sc.info.depth > SOLRT_BVH2_STACK) {
        set_error("BVH2 depth %u exceeds the traversal stack (%d)", sc.info.depth, SOLRT_BVH2_STACK);
        return SOLRT_ERR_CAPACITY;
    }
    return SOLRT_OK;
}

// ---------------------------------------------------------------------------
// Dynamic scenes (solrt_scene_set_instances + solrt_scene_regenerate): the
// per-frame instance transforms of SceneDescription::blas_transforms and
// tlas_regenerate (src/ray/mod.rs:162-181).
// ---------------------------------------------------------------------------

namespace {

// World-space position of vertex v (for the BVH) from its object-space copy
// and the instance of its section, with the operation order of
// solrt_scene_create (mat4_mul), so a regenerated scene equals one created
// with these instances bit for bit. Shading reads the instances directly.
__global__ void k_apply_instances(const float4* __restrict__ opos, const uint32_t* __restrict__ vsec_start,
                                  uint32_t nsec, const solrt_instance* __restrict__ inst, uint32_t nv,
                                  float4* __restrict__ vpos) {
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    // last section whose first vertex is <= v (empty sections share starts
    // with their successor and are skipped by taking the last)
    uint32_t lo = 0, hi = nsec - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (vsec_start[mid] <= v) lo = mid;
        else hi = mid - 1;
    }
    const solrt_instance& in = inst[lo];
    float o[4];
    const float4 p = opos[v];
    mat4_mul(in.transform, p.x, p.y, p.z, 1.0f, o);
    vpos[v] = make_float4(o[0], o[1], o[2], 0.0f);
}

// New boxes for the kept topology: the refit pass of build_bvh over the
// moved triangles, then (BVH8) a fresh collapse of the refitted tree.
solrt_status refit_bvh(Context& ctx, Scene& sc) {
    const uint32_t n = sc.tri_count;
    const uint32_t ni = n > 1 ? n - 1 : 1;
    cudaStream_t st = ctx.stream;
    SOLRT_CUDA(cudaEventRecord(ctx.ev0, st));
    const bool b8 = sc.info.kind == SOLRT_BVH8_Q8 || sc.info.kind == SOLRT_BVH4_Q8 || sc.info.kind == SOLRT_BVH8_F32;
    const uint32_t width = sc.info.kind == SOLRT_BVH4_Q8 ? 4u : 8u;
    const bool f32 = sc.info.kind == SOLRT_BVH8_F32;
    const bool q16 = sc.info.kind == SOLRT_BVH2_Q16;
    DeviceBuffer flags, nbox, nodes2, tri2;
    SOLRT_TRY(flags.alloc(sizeof(unsigned int) * (size_t)ni));
    SOLRT_TRY(nbox.alloc(2 * sizeof(float4) * (size_t)ni));
    float4* nodes_out = sc.nodes.as<float4>();
    float4* tri_out = sc.tri_wt.as<float4>();
    if (b8) {
        SOLRT_TRY(nodes2.alloc(4 * sizeof(float4) * (size_t)ni));
        SOLRT_TRY(tri2.alloc(3 * sizeof(float4) * (size_t)n));
        nodes_out = nodes2.as<float4>();
        tri_out = tri2.as<float4>();
    } else if (q16) {  // FP32 nodes first, quantised below
        SOLRT_TRY(nodes2.alloc(4 * sizeof(float4) * (size_t)ni));
        nodes_out = nodes2.as<float4>();
    }
    SOLRT_CUDA(cudaMemsetAsync(flags.ptr, 0, flags.bytes, st));
    k_refit<<<blocks_for(n, 256), 256, 0, st>>>(sc.vpos.as<float4>(), sc.tri_idx.as<uint4>(),
                                                sc.topo_order.as<uint32_t>(), sc.topo_child.as<uint32_t>(),
                                                sc.topo_par_int.as<uint32_t>(), sc.topo_par_leaf.as<uint32_t>(), n,
                                                flags.as<unsigned int>(), nbox.as<float4>(), nodes_out, tri_out);
    ++ctx.launches;
    SOLRT_CUDA(cudaGetLastError());
    if (b8) {
        Bvh8BuildInput in;
        in.n = n;
        in.child = sc.topo_child.as<uint32_t>();
        in.nbox = nbox.as<float4>();
        in.range = sc.topo_range.as<uint2>();
        in.tri_wt_leaf = tri2.as<float4>();
        in.leaf_max = sc.desc.leaf_max == 0 ? 1u : std::min(3u, sc.desc.leaf_max);
        in.par_int = sc.topo_par_int.as<uint32_t>();
        in.par_leaf = sc.topo_par_leaf.as<uint32_t>();
        in.sah = (sc.desc.flags & SOLRT_BVH_SAH) != 0;
        DeviceBuffer nodes8, tri8;
        uint32_t node_count = 0, depth8 = 0;
        SOLRT_TRY(build_wide(ctx, in, width, f32, nodes8, tri8, &node_count, &depth8));
        SOLRT_TRY(check_wide_depth(width, depth8));
        sc.nodes.adopt(nodes8);
        sc.tri_wt.adopt(tri8);
        sc.info.node_count = node_count;
        sc.info.depth = depth8;
        sc.info.node_bytes = (uint64_t)node_count * (width == 4 ? 64u : (f32 ? 224u : 80u));
        sc.info.tri_bytes = sc.tri_wt.bytes;
    } else if (q16) {
        SOLRT_TRY(quantize_bvh2(ctx, nodes2, nbox.as<float4>(), ni));
        sc.nodes.adopt(nodes2);
    }
    SOLRT_CUDA(cudaEventRecord(ctx.ev1, st));
    SOLRT_CUDA(cudaEventSynchronize(ctx.ev1));
    float ms = 0.0f;
    SOLRT_CUDA(cudaEventElapsedTime(&ms, ctx.ev0, ctx.ev1));
    sc.info.build_ms = ms;
    return SOLRT_OK;
}

}  // namespace

solrt_status regenerate_scene(Context& ctx, Scene& sc, uint32_t mode) {
    cudaGetLastError();  // launch errors below must be this call's own
    cudaStream_t st = ctx.stream;
    if (sc.vertex_count) {
        k_apply_instances<<<blocks_for(sc.vertex_count, 256), 256, 0, st>>>(
            sc.opos.as<float4>(), sc.vsec_start.as<uint32_t>(), sc.section_count, sc.instances.as<solrt_instance>(),
            sc.vertex_count, sc.vpos.as<float4>());
        ++ctx.launches;
        SOLRT_CUDA(cudaGetLastError());
    }
    if (sc.info.kind == SOLRT_BVH2_TWO_LEVEL) {  // BLASes stay; a new TLAS for the instances
        if (sc.tri_count == 0) return SOLRT_OK;
        SOLRT_CUDA(cudaEventRecord(ctx.ev0, st));
        SOLRT_TRY(build_tlas(ctx, sc));
        SOLRT_CUDA(cudaEventRecord(ctx.ev1, st));
        SOLRT_CUDA(cudaEventSynchronize(ctx.ev1));
        float ms = 0.0f;
        SOLRT_CUDA(cudaEventElapsedTime(&ms, ctx.ev0, ctx.ev1));
        sc.info.build_ms = ms;
        sc.info.depth = sc.blas_depth + sc.tlas_depth;
        return SOLRT_OK;
    }
    if (mode == SOLRT_REGEN_REFIT && sc.tri_count > 0 && sc.topo_order.ptr && sc.nodes.ptr)
        return refit_bvh(ctx, sc);
    return build_bvh(ctx, sc, sc.desc);
}

// ---------------------------------------------------------------------------
// Allocation-free BVH2 build (solrt_bvh2_build_noalloc): the same kernels as
// build_bvh, with their temporary arrays carved out of one fixed scratch
// array that is part of the library image instead of cudaMalloc'ed buffers.
// ---------------------------------------------------------------------------

namespace {

constexpr uint32_t kNoAllocTris = SOLRT_NOALLOC_MAX_TRIS;
constexpr uint32_t kNoAllocSortBlocks = (kNoAllocTris + kSortTile - 1) / kSortTile;
constexpr size_t round256(size_t x) { return (x + 255) & ~size_t(255); }

// Byte offsets of the temporary arrays inside the scratch array.
constexpr size_t kOffCen = 0;                                                      // float4 x n
constexpr size_t kOffCb = kOffCen + round256(16ull * kNoAllocTris);               // 6 x u32
constexpr size_t kOffKeys0 = kOffCb + 256;                                         // u32 x n
constexpr size_t kOffKeys1 = kOffKeys0 + round256(4ull * kNoAllocTris);
constexpr size_t kOffVals0 = kOffKeys1 + round256(4ull * kNoAllocTris);
constexpr size_t kOffVals1 = kOffVals0 + round256(4ull * kNoAllocTris);
constexpr size_t kOffHist = kOffVals1 + round256(4ull * kNoAllocTris);            // u32 x 256 x blocks
constexpr size_t kOffChild = kOffHist + round256(4ull * 256 * kNoAllocSortBlocks);  // u32 x 2(n-1)
constexpr size_t kOffParInt = kOffChild + round256(8ull * kNoAllocTris);
constexpr size_t kOffParLeaf = kOffParInt + round256(4ull * kNoAllocTris);
constexpr size_t kOffFlags = kOffParLeaf + round256(4ull * kNoAllocTris);
constexpr size_t kOffNbox = kOffFlags + round256(4ull * kNoAllocTris);             // 2 float4 x (n-1)
constexpr size_t kNoAllocBytes = kOffNbox + round256(32ull * kNoAllocTris);

}  // namespace

// Scratch of the allocation-free build. Host code must not use this name as a
// pointer (on the host it is only a stand-in): every call takes the device
// address from cudaGetSymbolAddress in the context current at that call.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {

// Device address of the scratch array in the current context. Looked up on
// every call and never cached: an address taken in one context is not valid
// in another (a host application's own context, or the primary context
// created again after cudaDeviceReset). The lookup is a host-side query
// that queues no GPU work.
solrt_status noalloc_scratch(void** out) {
    void* p = nullptr;
    SOLRT_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    *out = p;
    return SOLRT_OK;
}

}  // namespace

}  // namespace solrt

extern "C" solrt_status solrt_bvh2_build_noalloc(const void* vpos, const void* tri_idx, uint32_t tri_count,
                                                 void* nodes, size_t nodes_bytes, void* tris, size_t tris_bytes,
                                                 void* stream) {
    using namespace solrt;
    if (tri_count > kNoAllocTris) {
        set_error("solrt_bvh2_build_noalloc: %u triangles exceed the limit of %u", tri_count, kNoAllocTris);
        return SOLRT_ERR_CAPACITY;
    }
    if (tri_count == 0) return SOLRT_OK;
    const uint32_t n = tri_count;
    const uint32_t ni = n > 1 ? n - 1 : 1;
    if (!vpos || !tri_idx || !nodes || !tris) {
        set_error("solrt_bvh2_build_noalloc: null pointer");
        return SOLRT_ERR_INVALID;
    }
    if (nodes_bytes < 64ull * ni || tris_bytes < 48ull * n) {
        set_error("solrt_bvh2_build_noalloc: output buffers too small (%zu < %llu or %zu < %llu)", nodes_bytes,
                  64ull * ni, tris_bytes, 48ull * n);
        return SOLRT_ERR_INVALID;
    }
    if (((uintptr_t)vpos | (uintptr_t)tri_idx | (uintptr_t)nodes | (uintptr_t)tris) & 15u) {
        set_error("solrt_bvh2_build_noalloc: buffers must be 16-byte aligned");
        return SOLRT_ERR_INVALID;
    }
    cudaGetLastError();  // launch errors below must be this call's own
    void* base = nullptr;
    SOLRT_TRY(noalloc_scratch(&base));
    unsigned char* s = static_cast<unsigned char*>(base);
    float4* cen = reinterpret_cast<float4*>(s + kOffCen);
    unsigned int* cb = reinterpret_cast<unsigned int*>(s + kOffCb);
    uint32_t* keys[2] = {reinterpret_cast<uint32_t*>(s + kOffKeys0), reinterpret_cast<uint32_t*>(s + kOffKeys1)};
    uint32_t* vals[2] = {reinterpret_cast<uint32_t*>(s + kOffVals0), reinterpret_cast<uint32_t*>(s + kOffVals1)};
    uint32_t* hist = reinterpret_cast<uint32_t*>(s + kOffHist);
    uint32_t* child = reinterpret_cast<uint32_t*>(s + kOffChild);
    uint32_t* par_int = reinterpret_cast<uint32_t*>(s + kOffParInt);
    uint32_t* par_leaf = reinterpret_cast<uint32_t*>(s + kOffParLeaf);
    unsigned int* flags = reinterpret_cast<unsigned int*>(s + kOffFlags);
    float4* nbox = reinterpret_cast<float4*>(s + kOffNbox);
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    // The scratch keeps the previous call's contents: reset what must start
    // at a known value (bounds accumulators, arrival flags, parent links).
    SOLRT_CUDA(cudaMemsetAsync(cb, 0xff, 3 * sizeof(unsigned int), st));
    SOLRT_CUDA(cudaMemsetAsync(cb + 3, 0, 3 * sizeof(unsigned int), st));
    SOLRT_CUDA(cudaMemsetAsync(flags, 0, sizeof(unsigned int) * ni, st));
    SOLRT_CUDA(cudaMemsetAsync(par_int, 0xff, sizeof(uint32_t) * ni, st));

    const float4* vp = static_cast<const float4*>(vpos);
    const uint4* ti = static_cast<const uint4*>(tri_idx);
    const uint32_t nblocks = blocks_for(n, kSortTile);
    k_centroids<<<blocks_for(n, 256), 256, 0, st>>>(vp, ti, n, cen, cb);
    k_morton<<<blocks_for(n, 256), 256, 0, st>>>(cen, cb, n, keys[0], vals[0]);
    int cur = 0;
    for (int shift = 0; shift < 30; shift += 8) {
        k_radix_hist<<<nblocks, kSortThreads, 0, st>>>(keys[cur], n, shift, nblocks, hist);
        k_scan_exclusive<<<1, 1024, 0, st>>>(hist, 256 * nblocks);
        k_radix_scatter<<<nblocks, kSortThreads, 0, st>>>(keys[cur], vals[cur], keys[cur ^ 1], vals[cur ^ 1], hist, n,
                                                          shift, nblocks);
        cur ^= 1;
    }
    if (n > 1) k_karras<<<blocks_for(n - 1, 256), 256, 0, st>>>(keys[cur], n, child, par_int, par_leaf, nullptr);
    k_refit<<<blocks_for(n, 256), 256, 0, st>>>(vp, ti, vals[cur], child, par_int, par_leaf, n, flags, nbox,
                                                static_cast<float4*>(nodes), static_cast<float4*>(tris));
    SOLRT_CUDA(cudaGetLastError());
    return SOLRT_OK;
}
