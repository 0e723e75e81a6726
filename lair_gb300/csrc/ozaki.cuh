// FP64 Schur update on the FP16 tensor cores (Ozaki scheme, see ozaki.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

struct luhot_ctx;

namespace luhot {

// Workspace of ozaki_update for a trailing block of at most m rows and n
// columns: the FP16 digit slices of L21 and U12 and their exponents (at
// least 128 rows' worth).
size_t ozaki_workspace_bytes(int m, int n);
// The device has the shared memory and the driver the tensor-map encoder.
bool ozaki_available(luhot_ctx* ctx);
// a[r1..m, c1..n] -= a[r1..m, k0..k0+w] a[k0..k0+w, c1..n] for the row-major
// FP64 matrix a (lda), K = w in steps of 64; ws holds
// ozaki_workspace_bytes(m - r1, n - c1) bytes.  Asynchronous on `stream`.
int ozaki_update(luhot_ctx* ctx, double* a, int64_t lda, int k0, int w, int r1, int m, int c1, int n, void* ws,
                 cudaStream_t stream);
// U12 = L11^-1 A12 for the unit lower triangular L11 = a[k0.., k0..] (w x w,
// w <= 64) and A12 = a[k0..k0+w, c1..n] (at least 128 columns), computed as
// A12 - N A12 with N = I - L11^-1 on the tensor cores; ws as for
// ozaki_update(.., m >= 128, n - c1).  Asynchronous on `stream`.
int ozaki_trsm(luhot_ctx* ctx, double* a, int64_t lda, int k0, int w, int c1, int n, void* ws, cudaStream_t stream);

}  // namespace luhot
