// tma_host.cu -- host-side encoding of TMA tensor maps.
//
// cuTensorMapEncodeTiled is a driver-API function; it is fetched once through
// the runtime's driver entry-point query so the library does not have to link
// libcuda at build time.
#include <mutex>

#include <cudaTypedefs.h>

#include "tma.cuh"

namespace gopf {

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

bool encode_map_8b(CUtensorMap *map, const void *base, int rank, const unsigned long long *dims,
                   const unsigned long long *strides_bytes, const unsigned *box)
{
    PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
    if (!fn || rank < 1 || rank > 3 || !base) return false;
    if ((reinterpret_cast<uintptr_t>(base) & 15u) != 0) return false; // TMA needs a 16-byte aligned base
    cuuint64_t gd[3], gs[2];
    cuuint32_t bx[3], es[3] = {1, 1, 1};
    for (int i = 0; i < rank; ++i) {
        gd[i] = dims[i];
        bx[i] = box[i];
        if (bx[i] == 0 || bx[i] > 256 || bx[i] > gd[i]) return false;
    }
    if ((bx[0] * 8u) % 16u != 0) return false; // inner box extent: a multiple of 16 bytes
    for (int i = 0; i + 1 < rank; ++i) {
        gs[i] = strides_bytes[i];
        if (gs[i] % 16u != 0) return false;
    }
    const CUresult r =
        fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT64, (cuuint32_t)rank, const_cast<void *>(base), gd, gs, bx, es,
           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

} // namespace gopf
