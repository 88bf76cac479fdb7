// bvh8_build.cu — collapse of the binary LBVH into the 8-wide quantised BVH.
#include "bvh8.cuh"

namespace solrt {

solrt_status build_bvh8(Context& ctx, const Bvh8BuildInput& in, DeviceBuffer& nodes, DeviceBuffer& tris,
                        uint32_t* node_count, uint32_t* depth) {
    set_error("BVH8 build not available");
    return SOLRT_ERR_INVALID;
}

}  // namespace solrt
