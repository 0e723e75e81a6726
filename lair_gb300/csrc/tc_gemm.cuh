// Tensor-core (tcgen05) Schur update for the mixed-precision LU (see tc_gemm.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

struct luhot_ctx;

namespace luhot {

// kTcBF16x3: FP32-accurate products from three BF16 pieces per operand.
enum TcKind : int { kTcFP16 = 0, kTcBF16 = 1, kTcTF32 = 2, kTcBF16x3 = 3 };

// K of the operand copies padded to whole 128-byte TMA boxes.
int tc_kalloc(int kind, int w);
// Bytes of one operand copy with `rows` rows for panel width w.
size_t tc_operand_bytes(int kind, int rows, int w);

// A22 -= L21 U12 for the panel [k0, k0 + w) of the row-major FP32 matrix a
// (m x n, lda), through scaled low-precision copies of L21 and U12^T (aop,
// bop: tc_operand_bytes(kind, m or n, w) each) and 8 floats of scalars.
int tc_schur_update(luhot_ctx* ctx, int kind, float* a, int64_t lda, int k0, int w, int m, int n, void* aop,
                    void* bop, float* scal, cudaStream_t stream);
// The same on any block: a[r1..m, c1..n] -= a[r1..m, k0..k0+w] a[k0..k0+w, c1..n]
// (the operand copies must hold tc_operand_bytes(kind, m - r1 or n - c1, w)).
int tc_gemm_update(luhot_ctx* ctx, int kind, float* a, int64_t lda, int k0, int w, int r1, int m, int c1, int n,
                   void* aop, void* bop, float* scal, cudaStream_t stream);

}  // namespace luhot
