// Sync-free blocked triangular solve (see trsv.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace luhot {

struct DeviceStatus;

// Dynamic shared memory per CTA and grid size (number of 64-row blocks).
size_t trsv_syncfree_smem(size_t elem_bytes);
int trsv_syncfree_blocks(int n);

// op(A) x = b in place for nrhs columns of x (row-major, ldx); flags must hold
// trsv_syncfree_blocks(n) ints and ticket one int of device scratch (both
// cleared by this call); st supplies the wait limit and records a timeout.
// TA is the storage type of the factor (it may be narrower than T).
template <typename T, typename TA = T>
cudaError_t launch_trsv_syncfree(cudaStream_t stream, const TA* a, int64_t lda, T* x, int64_t ldx, int n, int nrhs,
                                 bool lower, bool unit, bool trans, bool exact, int* flags, int* ticket,
                                 DeviceStatus* st);

}  // namespace luhot
