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
// 4 * trsv_syncfree_blocks(n) ints and ticket one int of device scratch (both
// cleared by this call); st supplies the wait limit and records a timeout.
// TA is the storage type of the factor (it may be narrower than T).  dinv,
// when not null, holds the inverses of the 64 x 64 diagonal blocks of the
// triangle of A that the sweep reads (launch_trsv_invert_diag; for a
// transposed sweep the inverses of A's blocks, read transposed) and replaces
// the sequential diagonal solve by a matvec; it is ignored in exact mode.
template <typename T, typename TA = T>
cudaError_t launch_trsv_syncfree(cudaStream_t stream, const TA* a, int64_t lda, T* x, int64_t ldx, int n, int nrhs,
                                 bool lower, bool unit, bool trans, bool exact, int* flags, int* ticket,
                                 DeviceStatus* st, const T* dinv = nullptr);

// Block-scaled single-right-hand-side sweeps (trsv_scaled.cu).  W holds,
// for every off-diagonal 64 x 64 tile of L (below) and U (above) of an n x n
// row-major factor, D_I^-1 T(I, J) with D_I the tile row's diagonal block;
// launch_scale_blocks forms it from the factor and the diagonal inverses of
// L and U.  launch_trsv_scaled then runs y = T^-1 b for the lower (L) or upper
// (U) triangle with b contiguous and y strided (y must not alias b); xt is
// tagged-word scratch of trsv_scaled_tag_words(n) words, epoch a tag no word
// of xt holds yet, ticket one int (cleared by the call).
size_t trsv_scaled_tag_words(int n);
template <typename TA, typename TW>
cudaError_t launch_scale_blocks(cudaStream_t stream, const TA* a, int64_t lda, const double* dinv_l,
                                const double* dinv_u, TW* w, int64_t ldw, int n);
template <typename TW>
cudaError_t launch_trsv_scaled(cudaStream_t stream, const TW* w, int64_t ldw, const double* dinv, const double* b,
                               double* y, int64_t ldy, int n, bool lower, unsigned long long* xt, unsigned int epoch,
                               int* ticket, DeviceStatus* st);

// Elements of the diagonal-block inverses for order n.
size_t trsv_inverse_elems(int n);
// Inverses of the diagonal blocks of the unit lower (lower) or non-unit upper
// triangle of a row-major LU factor.
template <typename T, typename TA = T>
cudaError_t launch_trsv_invert_diag(cudaStream_t stream, const TA* a, int64_t lda, int n, bool lower, T* dinv);

// Chained sweep for one right-hand side with FP32 factors (trsv_chain.cu):
// 128-row blocks publishing x as epoch-tagged words.  dinv holds the inverses
// of the 128 x 128 diagonal blocks (launch_trsv_chain_invert); xt
// trsv_chain_tag_words(n) words of device scratch zeroed once, then reused
// with a new nonzero epoch per launch; ticket one int (cleared here).
int trsv_chain_blocks(int n);
size_t trsv_chain_inverse_elems(int n);
size_t trsv_chain_tag_words(int n);
template <typename T>
cudaError_t launch_trsv_chain_invert(cudaStream_t stream, const float* a, int64_t lda, int n, bool lower, T* dinv);
template <typename T>
cudaError_t launch_trsv_chain(cudaStream_t stream, const float* a, int64_t lda, T* x, int n, bool lower,
                              const T* dinv, unsigned long long* xt, unsigned int epoch, int* ticket,
                              DeviceStatus* st);

}  // namespace luhot
