// Sparse kernels shared by the solver sources.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "device.h"

namespace sucem {
cudaError_t spmv(const DeviceSpace& d, int dtype, const void* vals, const void* x, void* y,
                 cudaStream_t s);
cudaError_t spmv_raw(int64_t n, int64_t nnz, const int32_t* indptr, const int32_t* indices,
                     int dtype, const void* vals, const void* x, void* y, cudaStream_t s);
}  // namespace sucem
