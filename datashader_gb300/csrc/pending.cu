// pending.cu -- entry points declared in dsgb.h whose kernels are not built yet.
#include "dsgb_internal.cuh"
using namespace dsgb;
extern "C" int64_t dsgb_pyramid_tile_offset(int32_t zmin, int32_t z, int32_t tile_size) {
    int64_t off = 0;
    for (int32_t k = zmin; k < z; ++k) off += ((int64_t)1 << (2 * k)) * tile_size * tile_size;
    return off;
}
extern "C" int dsgb_pyramid(const dsgb_column *, int32_t, int64_t, int32_t, int32_t, int32_t,
                            const dsgb_pyramid_config *, uint32_t *, int64_t *, uint32_t, void *) {
    set_error("dsgb_pyramid: not built"); return DSGB_E_UNSUPPORTED;
}
extern "C" int dsgb_pyramid_finalize(const int64_t *, double *, int64_t, void *) {
    set_error("dsgb_pyramid_finalize: not built"); return DSGB_E_UNSUPPORTED;
}
