// tmap.cu -- host-side TMA descriptor encoding.
//
// cuTensorMapEncodeTiled is a driver API entry point; it is fetched through
// the runtime's driver-entry-point query so that libugemm_cuda.so needs no
// link-time dependency on libcuda (the library then loads on machines
// without a GPU, e.g. to check its exported symbols).
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "internal.h"

namespace ugemm {
namespace {

using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                              const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                              const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                              CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeFn get_encode() {
  static EncodeFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeFn>(p);
  });
  return fn;
}

bool encode(CUtensorMap* map, CUtensorMapDataType dtype, cuuint32_t rank, const void* base,
            const cuuint64_t* dims, const cuuint64_t* strides, const cuuint32_t* box,
            CUtensorMapSwizzle swz) {
  EncodeFn fn = get_encode();
  if (!fn) return false;
  cuuint32_t estr[3] = {1, 1, 1};
  return fn(map, dtype, rank, const_cast<void*>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

bool encode_tmap_2d(CUtensorMap* map, CUtensorMapDataType dtype, int /*elem_bytes*/,
                    const void* base, uint64_t inner, uint64_t outer, uint64_t row_bytes,
                    uint32_t box_inner, uint32_t box_outer, CUtensorMapSwizzle swz) {
  cuuint64_t dims[2] = {inner, outer};
  cuuint64_t strides[1] = {row_bytes};
  cuuint32_t box[2] = {box_inner, box_outer};
  return encode(map, dtype, 2, base, dims, strides, box, swz);
}

bool encode_tmap_3d(CUtensorMap* map, CUtensorMapDataType dtype, int /*elem_bytes*/,
                    const void* base, uint64_t d0, uint64_t d1, uint64_t d2, uint64_t stride1,
                    uint64_t stride2, uint32_t b0, uint32_t b1, uint32_t b2,
                    CUtensorMapSwizzle swz) {
  cuuint64_t dims[3] = {d0, d1, d2};
  cuuint64_t strides[2] = {stride1, stride2};
  cuuint32_t box[3] = {b0, b1, b2};
  return encode(map, dtype, 3, base, dims, strides, box, swz);
}

}  // namespace ugemm
