// tma.cu -- host side of the tensor maps (tma.cuh).
#include <cuda_runtime.h>

#include <mutex>

#include "tma.cuh"

namespace tma {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  });
  return fn;
}

bool encode_fields(CUtensorMap* out, const void* base, int elem_bytes, int n1m, int n2m, int n3m, int P,
                   size_t cells, int nfield, const int box[4]) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
  if (!fn || !base || (elem_bytes != 4 && elem_bytes != 8)) return false;
  if (((uintptr_t)base & 15) != 0) return false;
  const cuuint64_t dims[4] = {(cuuint64_t)n1m, (cuuint64_t)n2m, (cuuint64_t)n3m, (cuuint64_t)nfield};
  const cuuint64_t strides[3] = {(cuuint64_t)P * elem_bytes, (cuuint64_t)P * n2m * elem_bytes,
                                 (cuuint64_t)cells * elem_bytes};
  for (cuuint64_t s : strides)
    if (s % 16 != 0) return false;
  cuuint32_t bx[4];
  for (int d = 0; d < 4; ++d) {
    if (box[d] < 1 || box[d] > 256) return false;
    bx[d] = (cuuint32_t)box[d];
  }
  if ((bx[0] * elem_bytes) % 16 != 0) return false;
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  CUresult r = fn(out, elem_bytes == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4,
                  const_cast<void*>(base), dims, strides, bx, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

}  // namespace tma
