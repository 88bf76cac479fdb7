// bvh8_traverse.cuh — traversal of the 8-wide quantised BVH (bvh8.cuh).
#pragma once

#include "traverse.cuh"

namespace solrt {

template <bool kCount>
SOLRT_D void trace_bvh8(const DevScene& sc, float ox, float oy, float oz, float dx, float dy, float dz, float tmin,
                        float tmax, HitRec& best, TraceCounters& cnt, uint32_t& eflags) {
    best.t = tmax;
    best.prim = SOLRT_NO_HIT;
    best.u = 0.0f;
    best.v = 0.0f;
    eflags |= SOLRT_EFLAG_INDEX;
}

}  // namespace solrt
