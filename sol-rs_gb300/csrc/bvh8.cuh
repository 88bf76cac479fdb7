// bvh8.cuh — 8-wide BVH with 8-bit quantised child boxes (compressed wide
// BVH after Ylitie, Karras, Laine, HPG 2017), built by collapsing the binary
// LBVH. Node layout (80 B = 5 x 16 B):
//   w0: origin p.xyz (float)            | e.xyz (int8 exponents), imask (u8)
//   w1: child_base (u32), tri_base (u32), meta[0..7] (u8)
//   w2: qlo.x[0..7], qlo.y[0..7]        (u8)
//   w3: qlo.z[0..7], qhi.x[0..7]        (u8)
//   w4: qhi.y[0..7], qhi.z[0..7]        (u8)
// The full-precision variant (SOLRT_BVH8_F32, 224 B = 7 x 32 B) keeps the
// same slots, meta bytes and child / triangle bases:
//   w0: child_base, tri_base, meta[0..3], meta[4..7]    w1: imask, 0, 0, 0
//   then lo.x[8], hi.x[8], lo.y[8], hi.y[8], lo.z[8], hi.z[8] (float), each
//   child box widened outward by widen_lo / widen_hi.
// Child slot s decodes to lo = p + qlo * 2^e, hi = p + qhi * 2^e per axis;
// the build rounds outward so the decoded box contains the child exactly.
// meta[s]: 0 = empty; internal child = 0b001_xxxxx with xxxxx = 24 + s;
// leaf child with k triangles at offset o from tri_base = (2^k - 1) << 5 | o.
// Internal children of a node are stored contiguously from child_base in
// slot order; imask bit s marks an internal child.
#pragma once

#include "internal.h"

namespace solrt {

struct Bvh8BuildInput {
    uint32_t n;                // triangles
    const uint32_t* child;     // binary LBVH: 2 refs per internal node (leaf = 0x80000000 | pos)
    const float4* nbox;        // binary LBVH internal boxes: lo, hi as 2 float4
    const uint2* range;        // binary LBVH internal nodes: first, last leaf position
    const float4* tri_wt_leaf; // triangles in LBVH leaf order (3 float4 each)
    uint32_t leaf_max;         // max triangles per leaf child (1..3)
    const uint32_t* par_int;   // binary LBVH: parent of each internal node (SAH collapse)
    const uint32_t* par_leaf;  // binary LBVH: parent of each leaf (SAH collapse)
    bool sah;                  // SAH-optimal collapse instead of largest-child-first
};

// In-place exclusive scan of `len` u32 counts (bvh_build.cu).
void launch_scan_exclusive(uint32_t* data, uint32_t len, cudaStream_t stream);

// Writes the `width`-wide nodes (8: 80 B quantised or, with f32, 224 B full
// precision; 4: 64 B quantised) into `nodes` and the triangles in leaf order
// into `tris`. Synchronises.
solrt_status build_wide(Context& ctx, const Bvh8BuildInput& in, uint32_t width, bool f32, DeviceBuffer& nodes,
                        DeviceBuffer& tris, uint32_t* node_count, uint32_t* depth);

}  // namespace solrt
