// bvh8_build.cu — collapse of the binary LBVH into the 8-wide or 4-wide BVH
// with 8-bit quantised child boxes (layouts in bvh8.cuh and k_emit4).
//
// Level-synchronous and deterministic: each level is a list of tasks (one
// binary node -> one 8-wide node). Per task, one thread
//   1. gathers up to 8 children by repeatedly opening the child with the
//      largest surface area among those holding more than `leaf_max`
//      triangles (those cannot be leaves), or, with the SAH collapse, by
//      decoding the choices of a bottom-up dynamic program (k_sah_costs);
//   2. (after an exclusive scan of the internal-child and triangle counts of
//      all tasks of the level) assigns children to slots so that slot s
//      holds the child whose centre lies most in direction
//      ((s&1)?+x:-x, (s&2)?+y:-y, (s&4)?+z:-z) from the node centre, greedily
//      by lowest cost; a ray of octant o then visits slots in the order of
//      s ^ o, roughly near to far;
//   3. quantises the child boxes outward on a power-of-two grid anchored
//      just below the node's minimum corner (widen_lo), with one extra grid
//      step of margin on every face that is not the anchor plane;
//   4. writes the node, the next level's tasks and the leaf triangles.
// Offsets come from scans, not atomics, so the output does not depend on
// thread scheduling.
#include <algorithm>
#include <cmath>
#include <vector>

#include "bvh8.cuh"

namespace solrt {

namespace {

constexpr uint32_t kLeafFlag = 0x80000000u;

struct Box3 {
    float lo[3], hi[3];
};

__device__ __forceinline__ Box3 ref_box(uint32_t ref, const float4* __restrict__ nbox,
                                        const float4* __restrict__ tris) {
    Box3 b;
    if (ref & kLeafFlag) {
        const uint32_t k = ref & ~kLeafFlag;
        const float4 a = tris[3 * (size_t)k], c = tris[3 * (size_t)k + 1], d = tris[3 * (size_t)k + 2];
        b.lo[0] = fminf(fminf(a.x, c.x), d.x); b.hi[0] = fmaxf(fmaxf(a.x, c.x), d.x);
        b.lo[1] = fminf(fminf(a.y, c.y), d.y); b.hi[1] = fmaxf(fmaxf(a.y, c.y), d.y);
        b.lo[2] = fminf(fminf(a.z, c.z), d.z); b.hi[2] = fmaxf(fmaxf(a.z, c.z), d.z);
    } else {
        const float4 l = nbox[2 * (size_t)ref], h = nbox[2 * (size_t)ref + 1];
        b.lo[0] = l.x; b.lo[1] = l.y; b.lo[2] = l.z;
        b.hi[0] = h.x; b.hi[1] = h.y; b.hi[2] = h.z;
    }
    return b;
}

__device__ __forceinline__ uint32_t ref_count(uint32_t ref, const uint2* __restrict__ range) {
    if (ref & kLeafFlag) return 1u;
    const uint2 r = range[ref];
    return r.y - r.x + 1u;
}

__device__ __forceinline__ uint32_t ref_first(uint32_t ref, const uint2* __restrict__ range) {
    return (ref & kLeafFlag) ? (ref & ~kLeafFlag) : range[ref].x;
}

__device__ __forceinline__ float half_area(const Box3& b) {
    const float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    return dx * dy + dy * dz + dz * dx;
}

// SAH-optimal collapse (after Ylitie, Karras and Laine, HPG 2017, section
// 4.1). For every binary node n and i = 1..W, cost(n, i) is the least SAH
// cost of representing n's subtree by at most i children of the wide node
// above it:
//   a subtree of <= leaf_max triangles is one leaf child:
//       cost(n, i) = A(n) * kSahTri * count(n)
//   otherwise (cost(n, 1): n becomes a wide node itself)
//       cost(n, 1) = A(n) * kSahNode + D(n, W)
//       cost(n, i) = min(cost(n, i - 1), D(n, i))
//   D(n, j) = min over k = 1..j-1 of cost(left, k) + cost(right, j - k)
// with A the half surface area. Nodes are finished bottom-up as in the refit
// (the second thread to arrive computes the node). Per internal node the
// table keeps cost(n, 1..W), the split k of each i (0: same as i - 1) in
// nibbles, and the split of D(n, W).
constexpr float kSahNode = 1.0f;
constexpr float kSahTri = 0.3f;

__device__ __forceinline__ float sah_leaf_cost(uint32_t ref, const uint2* __restrict__ range,
                                               const float4* __restrict__ nbox, const float4* __restrict__ tris) {
    return half_area(ref_box(ref, nbox, tris)) * kSahTri * (float)ref_count(ref, range);
}

__global__ void k_sah_costs(uint32_t n, const uint32_t* __restrict__ child, const uint32_t* __restrict__ par_int,
                            const uint32_t* __restrict__ par_leaf, const uint2* __restrict__ range,
                            const float4* __restrict__ nbox, const float4* __restrict__ tris, uint32_t leaf_max,
                            uint32_t width, unsigned int* __restrict__ flags, float* __restrict__ cost,
                            uint2* __restrict__ dec) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || n < 2) return;
    const int W = (int)width;
    uint32_t p = par_leaf[k];
    for (uint32_t steps = 0; steps < n; ++steps) {
        if (p >= n - 1) return;  // malformed parent link: stop
        __threadfence();
        if (atomicAdd(flags + p, 1u) == 0u) return;
        __threadfence();
        float c[8];
        uint32_t decs = 0, dw = 0;
        const float area = half_area(ref_box(p, nbox, tris));
        if (ref_count(p, range) <= leaf_max) {
            const float lc = area * kSahTri * (float)ref_count(p, range);
            for (int i = 0; i < 8; ++i) c[i] = lc;
        } else {
            float cl[8], cr[8];
            for (int side = 0; side < 2; ++side) {
                const uint32_t r = child[2 * (size_t)p + side];
                float* t = side ? cr : cl;
                if ((r & kLeafFlag) || ref_count(r, range) <= leaf_max) {
                    const float lc = sah_leaf_cost(r, range, nbox, tris);
                    for (int i = 0; i < 8; ++i) t[i] = lc;
                } else {
                    for (int i = 0; i < 8; ++i) t[i] = __ldcg(cost + 8 * (size_t)r + i);
                }
            }
            float D[9];
            uint32_t K[9];
            for (int j = 2; j <= W; ++j) {
                D[j] = INFINITY;
                K[j] = 1;
                for (int s = 1; s < j; ++s) {
                    const float v = cl[s - 1] + cr[j - s - 1];
                    if (v < D[j]) { D[j] = v; K[j] = (uint32_t)s; }
                }
            }
            c[0] = area * kSahNode + D[W];
            dw = K[W];
            for (int i = 2; i <= W; ++i) {
                if (D[i] < c[i - 2]) {
                    c[i - 1] = D[i];
                    decs |= K[i] << (4 * (i - 1));
                } else {
                    c[i - 1] = c[i - 2];
                }
            }
            for (int i = W; i < 8; ++i) c[i] = c[W - 1];
        }
        for (int i = 0; i < 8; ++i) __stcg(cost + 8 * (size_t)p + i, c[i]);
        __stcg(dec + p, make_uint2(decs, dw));
        if (p == 0) return;
        p = par_int[p];
    }
}

// The children of wide node `b` chosen by the SAH collapse: D(b, W)'s split,
// each side resolved to the roots of its cost(r, i) choice.
__device__ int sah_children(uint32_t b, uint32_t width, const uint32_t* __restrict__ child,
                            const uint2* __restrict__ range, uint32_t leaf_max, const uint2* __restrict__ dec,
                            uint32_t* c) {
    uint32_t sr[16];
    uint32_t si[16];
    int sp = 0, m = 0;
    const uint32_t k = dec[b].y;
    sr[sp] = child[2 * (size_t)b + 1]; si[sp++] = width - k;
    sr[sp] = child[2 * (size_t)b]; si[sp++] = k;
    while (sp > 0 && m < 8) {
        const uint32_t r = sr[--sp];
        uint32_t i = si[sp];
        if ((r & kLeafFlag) || ref_count(r, range) <= leaf_max) {
            c[m++] = r;
            continue;
        }
        const uint32_t decs = dec[r].x;
        while (i > 1 && ((decs >> (4 * (i - 1))) & 15u) == 0u) --i;
        if (i <= 1 || sp + 2 > 16) {
            c[m++] = r;
            continue;
        }
        const uint32_t s = (decs >> (4 * (i - 1))) & 15u;
        sr[sp] = child[2 * (size_t)r + 1]; si[sp++] = i - s;
        sr[sp] = child[2 * (size_t)r]; si[sp++] = s;
    }
    return m;
}

// Pass 1: gather children, count internal children and leaf triangles.
__global__ void k_gather(const uint32_t* __restrict__ tasks, uint32_t ntasks, const uint32_t* __restrict__ child,
                         const uint2* __restrict__ range, const float4* __restrict__ nbox,
                         const float4* __restrict__ tris, uint32_t leaf_max, uint32_t width,
                         const uint2* __restrict__ sah_dec, uint32_t* __restrict__ gathered,
                         uint32_t* __restrict__ n_inner, uint32_t* __restrict__ n_tris) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t > ntasks) return;
    if (t == ntasks) {  // trailing zero so the exclusive scans end with the totals
        n_inner[t] = 0;
        n_tris[t] = 0;
        return;
    }
    const uint32_t b = tasks[t];
    uint32_t c[8];
    int m;
    if (b & kLeafFlag) {  // single-triangle scene: the root holds one leaf
        c[0] = b;
        m = 1;
    } else if (sah_dec) {
        m = sah_children(b, width, child, range, leaf_max, sah_dec, c);
    } else {
        c[0] = child[2 * (size_t)b];
        c[1] = child[2 * (size_t)b + 1];
        m = 2;
        while (m < (int)width) {
            int best = -1;
            float best_a = -1.0f;
            for (int i = 0; i < m; ++i) {
                if ((c[i] & kLeafFlag) || ref_count(c[i], range) <= leaf_max) continue;
                const float a = half_area(ref_box(c[i], nbox, tris));
                if (a > best_a) { best_a = a; best = i; }
            }
            if (best < 0) break;
            const uint32_t r = c[best];
            c[best] = child[2 * (size_t)r];
            c[m++] = child[2 * (size_t)r + 1];
        }
    }
    uint32_t inner = 0, ntri = 0;
    for (int i = 0; i < 8; ++i) {
        const uint32_t r = i < m ? c[i] : 0xffffffffu;
        gathered[8 * (size_t)t + i] = r;
        if (i < m) {
            const uint32_t k = ref_count(r, range);
            if (k > leaf_max) ++inner;
            else ntri += k;
        }
    }
    n_inner[t] = inner;
    n_tris[t] = ntri;
}

// Smallest e with ext / 2^e <= limit, clamped to [-126, 127].
__device__ __forceinline__ int grid_exponent(double ext, double limit) {
    const double x = ext / limit;
    if (!(x > 0.0)) return -126;
    int k = 0;
    const double m = frexp(x, &k);  // x = m * 2^k, m in [0.5, 1)
    int e = (m == 0.5) ? k - 1 : k;
    // x was rounded: make sure the grid really spans ext (scaling is exact)
    while (e < 127 && ext * ldexp(1.0, -e) > limit) ++e;
    return e < -126 ? -126 : (e > 127 ? 127 : e);
}

// Anchor of a node's grid on one axis: one grid step below widen_lo(lo),
// rounded down to a float, with the exponent raised until hi is within 253
// steps. Every decoded face, q = 0 included, then lies at least one step
// outside the child it bounds (q ranges over 0..255 with the +-1 margins).
__device__ __forceinline__ void grid_anchor(float lo, float hi, float& p, int& e) {
    const float p0 = widen_lo(lo);
    e = grid_exponent((double)hi - (double)p0, 252.0);
    for (;;) {
        const double pd = (double)p0 - ldexp(1.0, e);
        float pf = (float)pd;
        if ((double)pf > pd) pf = nextafterf(pf, -INFINITY);
        p = pf;
        if (e >= 127 || ((double)hi - (double)pf) * ldexp(1.0, -e) <= 253.0) break;
        ++e;
    }
}

// Pass 2: slots, quantisation, node + next tasks + leaf triangles.
// f32: write the full-precision 224-byte node (header + 6 x 8 FP32 planes,
// each child box widened outward by widen_lo / widen_hi) instead of the
// quantised 80-byte one.
__global__ void k_emit(const uint32_t* __restrict__ tasks, uint32_t ntasks, uint32_t node_base,
                       uint32_t next_base, uint32_t tri_level_base, const uint32_t* __restrict__ gathered,
                       const uint32_t* __restrict__ inner_scan, const uint32_t* __restrict__ tri_scan,
                       const uint2* __restrict__ range, const float4* __restrict__ nbox,
                       const float4* __restrict__ tris_in, uint32_t leaf_max, uint4* __restrict__ nodes,
                       uint32_t* __restrict__ next_tasks, float4* __restrict__ tris_out, bool f32) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntasks) return;
    const uint32_t b = tasks[t];
    Box3 cb[8];
    uint32_t cr[8];
    int m = 0;
    for (int i = 0; i < 8; ++i) {
        const uint32_t r = gathered[8 * (size_t)t + i];
        if (r == 0xffffffffu) break;
        cr[m] = r;
        cb[m] = ref_box(r, nbox, tris_in);
        ++m;
    }
    // node box = union of the children
    Box3 nb = cb[0];
    for (int i = 1; i < m; ++i)
        for (int a = 0; a < 3; ++a) {
            nb.lo[a] = fminf(nb.lo[a], cb[i].lo[a]);
            nb.hi[a] = fmaxf(nb.hi[a], cb[i].hi[a]);
        }
    // slot assignment
    int slot_of[8];
    int child_in_slot[8];
    for (int i = 0; i < 8; ++i) { slot_of[i] = -1; child_in_slot[i] = -1; }
    float cost[8][8];
    for (int i = 0; i < m; ++i) {
        float off[3];
        for (int a = 0; a < 3; ++a)
            off[a] = (cb[i].lo[a] + cb[i].hi[a]) - (nb.lo[a] + nb.hi[a]);
        for (int s = 0; s < 8; ++s) {
            const float dx = (s & 1) ? off[0] : -off[0];
            const float dy = (s & 2) ? off[1] : -off[1];
            const float dz = (s & 4) ? off[2] : -off[2];
            cost[i][s] = -((dx + dy) + dz);
        }
    }
    for (int step = 0; step < m; ++step) {
        int bi = -1, bs = -1;
        float bc = 0.0f;
        for (int i = 0; i < m; ++i) {
            if (slot_of[i] >= 0) continue;
            for (int s = 0; s < 8; ++s) {
                if (child_in_slot[s] >= 0) continue;
                if (bi < 0 || cost[i][s] < bc) { bi = i; bs = s; bc = cost[i][s]; }
            }
        }
        slot_of[bi] = bs;
        child_in_slot[bs] = bi;
    }
    // grid
    int e[3];
    float p[3];
    for (int a = 0; a < 3; ++a) grid_anchor(nb.lo[a], nb.hi[a], p[a], e[a]);
    uint32_t qlo[3][2] = {{0, 0}, {0, 0}, {0, 0}}, qhi[3][2] = {{0, 0}, {0, 0}, {0, 0}};
    uint32_t meta[2] = {0, 0};
    uint32_t imask = 0;
    const uint32_t child_base = next_base + inner_scan[t];
    const uint32_t tri_base = tri_level_base + tri_scan[t];
    uint32_t inner_rank = 0, tri_off = 0;
    for (int s = 0; s < 8; ++s) {
        const int i = child_in_slot[s];
        if (i < 0) continue;
        for (int a = 0; a < 3; ++a) {
            const double inv_step = ldexp(1.0, -e[a]);
            // Outward rounding plus one grid step of margin on every face:
            // a decoded face never lies within one step of the child's
            // triangles (the anchor sits one step below the node's box, so
            // the low clamp below does not bind).
            const double lr = ((double)cb[i].lo[a] - (double)p[a]) * inv_step;
            const double hr = ((double)cb[i].hi[a] - (double)p[a]) * inv_step;
            double ql = floor(lr) - 1.0;
            double qh = ceil(hr) + 1.0;
            ql = ql < 0.0 ? 0.0 : ql;
            qh = qh > 255.0 ? 255.0 : qh;
            const uint32_t sh = 8u * (uint32_t)(s & 3);
            qlo[a][s >> 2] |= (uint32_t)ql << sh;
            qhi[a][s >> 2] |= (uint32_t)qh << sh;
        }
        const uint32_t r = cr[i];
        const uint32_t k = ref_count(r, range);
        uint32_t mb;
        if (k > leaf_max) {
            imask |= 1u << s;
            mb = (1u << 5) | (24u + (uint32_t)s);
            next_tasks[inner_scan[t] + inner_rank] = r;
            ++inner_rank;
        } else {
            mb = (((1u << k) - 1u) << 5) | tri_off;
            const uint32_t first = ref_first(r, range);
            for (uint32_t j = 0; j < k; ++j) {
                const size_t src = 3 * (size_t)(first + j), dst = 3 * (size_t)(tri_base + tri_off + j);
                tris_out[dst] = tris_in[src];
                tris_out[dst + 1] = tris_in[src + 1];
                tris_out[dst + 2] = tris_in[src + 2];
            }
            tri_off += k;
        }
        meta[s >> 2] |= mb << (8u * (uint32_t)(s & 3));
    }
    if (f32) {
        uint4* out = nodes + 14 * (size_t)(node_base + t);
        out[0] = make_uint4(child_base, tri_base, meta[0], meta[1]);
        out[1] = make_uint4(imask, 0u, 0u, 0u);
        float* planes = reinterpret_cast<float*>(out + 2);  // [axis][lo / hi][slot]
        for (int s = 0; s < 8; ++s) {
            const int i = child_in_slot[s];
            for (int a = 0; a < 3; ++a) {
                planes[(2 * a) * 8 + s] = i < 0 ? 0.0f : widen_lo(cb[i].lo[a]);
                planes[(2 * a + 1) * 8 + s] = i < 0 ? 0.0f : widen_hi(cb[i].hi[a]);
            }
        }
        return;
    }
    const uint32_t packed = ((uint32_t)(uint8_t)(int8_t)e[0]) | ((uint32_t)(uint8_t)(int8_t)e[1] << 8) |
                            ((uint32_t)(uint8_t)(int8_t)e[2] << 16) | (imask << 24);
    uint4* out = nodes + 5 * (size_t)(node_base + t);
    out[0] = make_uint4(__float_as_uint(p[0]), __float_as_uint(p[1]), __float_as_uint(p[2]), packed);
    out[1] = make_uint4(child_base, tri_base, meta[0], meta[1]);
    out[2] = make_uint4(qlo[0][0], qlo[0][1], qlo[1][0], qlo[1][1]);
    out[3] = make_uint4(qlo[2][0], qlo[2][1], qhi[0][0], qhi[0][1]);
    out[4] = make_uint4(qhi[1][0], qhi[1][1], qhi[2][0], qhi[2][1]);
}

// Pass 2 of the 4-wide collapse: quantisation as k_emit, slots in gathered
// order (the traversal orders hit children by distance), 64-byte nodes:
//   w0: origin p.xyz (float) | e.xyz (int8), imask (low 4 bits of the top byte)
//   w1: child_base, tri_base, meta[0..3] (u8), qlo.x[0..3] (u8)
//   w2: qlo.y[0..3], qlo.z[0..3], qhi.x[0..3], qhi.y[0..3]
//   w3: qhi.z[0..3], 0, 0, 0
__global__ void k_emit4(const uint32_t* __restrict__ tasks, uint32_t ntasks, uint32_t node_base,
                        uint32_t next_base, uint32_t tri_level_base, const uint32_t* __restrict__ gathered,
                        const uint32_t* __restrict__ inner_scan, const uint32_t* __restrict__ tri_scan,
                        const uint2* __restrict__ range, const float4* __restrict__ nbox,
                        const float4* __restrict__ tris_in, uint32_t leaf_max, uint4* __restrict__ nodes,
                        uint32_t* __restrict__ next_tasks, float4* __restrict__ tris_out) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntasks) return;
    Box3 cb[4];
    uint32_t cr[4];
    int m = 0;
    for (int i = 0; i < 4; ++i) {
        const uint32_t r = gathered[8 * (size_t)t + i];
        if (r == 0xffffffffu) break;
        cr[m] = r;
        cb[m] = ref_box(r, nbox, tris_in);
        ++m;
    }
    Box3 nb = cb[0];
    for (int i = 1; i < m; ++i)
        for (int a = 0; a < 3; ++a) {
            nb.lo[a] = fminf(nb.lo[a], cb[i].lo[a]);
            nb.hi[a] = fmaxf(nb.hi[a], cb[i].hi[a]);
        }
    int e[3];
    float p[3];
    for (int a = 0; a < 3; ++a) grid_anchor(nb.lo[a], nb.hi[a], p[a], e[a]);
    uint32_t qlo[3] = {0, 0, 0}, qhi[3] = {0, 0, 0};
    uint32_t meta = 0, imask = 0;
    const uint32_t child_base = next_base + inner_scan[t];
    const uint32_t tri_base = tri_level_base + tri_scan[t];
    uint32_t inner_rank = 0, tri_off = 0;
    for (int s = 0; s < m; ++s) {
        for (int a = 0; a < 3; ++a) {
            const double inv_step = ldexp(1.0, -e[a]);
            // outward rounding + one grid step of margin (see k_emit)
            const double lr = ((double)cb[s].lo[a] - (double)p[a]) * inv_step;
            const double hr = ((double)cb[s].hi[a] - (double)p[a]) * inv_step;
            double ql = floor(lr) - 1.0;
            double qh = ceil(hr) + 1.0;
            ql = ql < 0.0 ? 0.0 : ql;
            qh = qh > 255.0 ? 255.0 : qh;
            qlo[a] |= (uint32_t)ql << (8u * (uint32_t)s);
            qhi[a] |= (uint32_t)qh << (8u * (uint32_t)s);
        }
        const uint32_t r = cr[s];
        const uint32_t k = ref_count(r, range);
        uint32_t mb;
        if (k > leaf_max) {
            imask |= 1u << s;
            mb = 1u << 5;
            next_tasks[inner_scan[t] + inner_rank] = r;
            ++inner_rank;
        } else {
            mb = (((1u << k) - 1u) << 5) | tri_off;
            const uint32_t first = ref_first(r, range);
            for (uint32_t j = 0; j < k; ++j) {
                const size_t src = 3 * (size_t)(first + j), dst = 3 * (size_t)(tri_base + tri_off + j);
                tris_out[dst] = tris_in[src];
                tris_out[dst + 1] = tris_in[src + 1];
                tris_out[dst + 2] = tris_in[src + 2];
            }
            tri_off += k;
        }
        meta |= mb << (8u * (uint32_t)s);
    }
    const uint32_t packed = ((uint32_t)(uint8_t)(int8_t)e[0]) | ((uint32_t)(uint8_t)(int8_t)e[1] << 8) |
                            ((uint32_t)(uint8_t)(int8_t)e[2] << 16) | (imask << 24);
    uint4* out = nodes + 4 * (size_t)(node_base + t);
    out[0] = make_uint4(__float_as_uint(p[0]), __float_as_uint(p[1]), __float_as_uint(p[2]), packed);
    out[1] = make_uint4(child_base, tri_base, meta, qlo[0]);
    out[2] = make_uint4(qlo[1], qlo[2], qhi[0], qhi[1]);
    out[3] = make_uint4(qhi[2], 0u, 0u, 0u);
}

inline uint32_t blocks_of(uint64_t n, uint32_t b) { return (uint32_t)((n + b - 1) / b); }

}  // namespace

solrt_status build_wide(Context& ctx, const Bvh8BuildInput& in, uint32_t width, bool f32, DeviceBuffer& nodes,
                        DeviceBuffer& tris, uint32_t* node_count, uint32_t* depth) {
    const uint32_t n = in.n;
    cudaStream_t st = ctx.stream;
    const uint32_t max_nodes = std::max(1u, n);
    SOLRT_TRY(nodes.alloc((width == 4 ? 64ull : (f32 ? 224ull : 80ull)) * max_nodes));
    SOLRT_TRY(tris.alloc(48ull * n));
    DeviceBuffer task[2], gathered, inner, ntri;
    SOLRT_TRY(task[0].alloc(4ull * max_nodes));
    SOLRT_TRY(task[1].alloc(4ull * max_nodes));
    SOLRT_TRY(gathered.alloc(32ull * max_nodes));
    SOLRT_TRY(inner.alloc(4ull * (max_nodes + 1)));
    SOLRT_TRY(ntri.alloc(4ull * (max_nodes + 1)));
    const uint32_t root = n > 1 ? 0u : kLeafFlag;  // binary root, or the single leaf
    SOLRT_CUDA(cudaMemcpyAsync(task[0].ptr, &root, 4, cudaMemcpyHostToDevice, st));
    DeviceBuffer sah_cost, sah_dec, sah_flags;
    const bool sah = in.sah && n > 1 && in.par_int && in.par_leaf;
    if (sah) {
        SOLRT_TRY(sah_cost.alloc(32ull * (n - 1)));
        SOLRT_TRY(sah_dec.alloc(8ull * (n - 1)));
        SOLRT_TRY(sah_flags.alloc(4ull * (n - 1)));
        SOLRT_CUDA(cudaMemsetAsync(sah_flags.ptr, 0, sah_flags.bytes, st));
        k_sah_costs<<<blocks_of(n, 256), 256, 0, st>>>(n, in.child, in.par_int, in.par_leaf, in.range, in.nbox,
                                                       in.tri_wt_leaf, in.leaf_max, width,
                                                       sah_flags.as<unsigned int>(), sah_cost.as<float>(),
                                                       sah_dec.as<uint2>());
        ++ctx.launches;
    }
    uint32_t ntasks = 1, node_base = 0, tri_level_base = 0, levels = 0;
    int cur = 0;
    while (ntasks > 0) {
        if (node_base + ntasks > max_nodes) {
            set_error("wide BVH collapse overflowed its node bound");
            return SOLRT_ERR_CAPACITY;
        }
        k_gather<<<blocks_of(ntasks + 1, 128), 128, 0, st>>>(task[cur].as<uint32_t>(), ntasks, in.child, in.range,
                                                             in.nbox, in.tri_wt_leaf, in.leaf_max, width,
                                                             sah ? sah_dec.as<uint2>() : nullptr,
                                                             gathered.as<uint32_t>(), inner.as<uint32_t>(),
                                                             ntri.as<uint32_t>());
        launch_scan_exclusive(inner.as<uint32_t>(), ntasks + 1, st);
        launch_scan_exclusive(ntri.as<uint32_t>(), ntasks + 1, st);
        uint32_t totals[2] = {0, 0};
        SOLRT_CUDA(cudaMemcpyAsync(&totals[0], inner.as<uint32_t>() + ntasks, 4, cudaMemcpyDeviceToHost, st));
        SOLRT_CUDA(cudaMemcpyAsync(&totals[1], ntri.as<uint32_t>() + ntasks, 4, cudaMemcpyDeviceToHost, st));
        const uint32_t next_base = node_base + ntasks;
        if (width == 4)
            k_emit4<<<blocks_of(ntasks, 128), 128, 0, st>>>(task[cur].as<uint32_t>(), ntasks, node_base, next_base,
                                                            tri_level_base, gathered.as<uint32_t>(),
                                                            inner.as<uint32_t>(), ntri.as<uint32_t>(), in.range,
                                                            in.nbox, in.tri_wt_leaf, in.leaf_max, nodes.as<uint4>(),
                                                            task[cur ^ 1].as<uint32_t>(), tris.as<float4>());
        else
            k_emit<<<blocks_of(ntasks, 128), 128, 0, st>>>(task[cur].as<uint32_t>(), ntasks, node_base, next_base,
                                                           tri_level_base, gathered.as<uint32_t>(),
                                                           inner.as<uint32_t>(), ntri.as<uint32_t>(), in.range,
                                                           in.nbox, in.tri_wt_leaf, in.leaf_max, nodes.as<uint4>(),
                                                           task[cur ^ 1].as<uint32_t>(), tris.as<float4>(), f32);
        ctx.launches += 4;
        SOLRT_CUDA(cudaStreamSynchronize(st));
        SOLRT_CUDA(cudaGetLastError());
        ++levels;
        node_base = next_base;
        tri_level_base += totals[1];
        ntasks = totals[0];
        cur ^= 1;
        if (levels > 4096) {
            set_error("wide BVH collapse did not terminate");
            return SOLRT_ERR_DEVICE;
        }
    }
    if (tri_level_base != n) {
        set_error("wide BVH collapse placed %u of %u triangles", tri_level_base, n);
        return SOLRT_ERR_DEVICE;
    }
    *node_count = node_base;
    *depth = levels;
    return SOLRT_OK;
}

}  // namespace solrt
