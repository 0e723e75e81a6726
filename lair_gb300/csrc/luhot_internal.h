// Internal declarations shared by the luhot translation units.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "luhot.h"

namespace luhot {

struct DeviceStatus;

constexpr int kMaxPanelCtas = 256;     // >= SM count
constexpr int kDefaultPanelWidth = 64; // FP64 / FP32 CUDA-core and DMMA paths
constexpr int kTcPanelWidth = 128;     // tensor-core (tcgen05) Schur-update path
constexpr int kMaxPanelWidth = 128;    // sizes the panel kernel's scratch
// Panel exchange slots: per step parity and CTA, an 8-word header (FP32:
// signed pivot key at 0, row id at 1, the candidate's next-column value at 2;
// FP64: key at 0-1, id at 2, next-column value at 3-4) and the candidate row
// segment from word 8, in 8-byte words of (payload, step tag), two words per
// FP64 value.
constexpr int kPanelHeaderWords = 8;
constexpr int kPanelSlotWords = kPanelHeaderWords + 2 * kMaxPanelWidth;
static_assert(kPanelSlotWords % 4 == 0, "panel slots are whole 32-byte sectors (32-byte header loads)");
constexpr size_t kPanelSlotBytes = 2 * (size_t)kMaxPanelCtas * kPanelSlotWords * sizeof(unsigned long long);
// Followed by the panel's row moves: up to 2 * kMaxPanelWidth (destination,
// source) pairs and their count.
constexpr size_t kPanelMovesBytes = (4 * (size_t)kMaxPanelWidth + 64) * sizeof(int);
constexpr size_t kPanelScratchBytes = kPanelSlotBytes + kPanelMovesBytes;
// Scalars the refinement keeps on the device and reads back (norms and one
// column of the GMRES Hessenberg matrix): this many doubles on each side.
constexpr int kIrScalarSlots = 512;

// Grow-only device buffer.
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
};

// Kernel classes for the optional CUDA-event profile.
enum ProfClass : int {
  kProfPanel = 0,
  kProfLaswp = 1,
  kProfTrsm = 2,
  kProfGemm = 3,
  kProfTrsv = 4,
  kProfPermute = 5,
  kProfRefine = 6,
  kProfOther = 7,
  kProfClasses = 8,
};

struct ProfRecord {
  int cls;
  cudaEvent_t start, stop;
  double flops, bytes;
};

}  // namespace luhot

struct luhot_ctx {
  int device = 0;
  int num_sms = 0;
  int max_smem_optin = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  std::mutex mu;
  std::string last_error;
  luhot::DeviceStatus* d_status = nullptr;
  luhot::DeviceStatus* h_status = nullptr;  // pinned mirror
  void* panel_scratch = nullptr;            // candidates of the panel kernel
  luhot::DevBuf work[4];                    // matrix / rhs / solution / misc
  luhot::DevBuf piv_buf;                    // int32 pivots
  luhot::DevBuf perm_buf;                   // int32 permutation
  luhot::DevBuf trsv_buf;                   // ready flags + ticket of the triangular sweeps
  luhot::DevBuf ir_buf[4];                  // refinement: low-precision LU, vectors, indices, rhs
  luhot::DevBuf adj_buf;                    // adjoint: A^T or dA
  luhot::DevBuf tc_buf;                     // tensor-core LU: operand copies + scales
  luhot::DevBuf dinv_buf;                   // inverses of the 64 x 64 diagonal blocks of L and U
  luhot::DevBuf chain_buf;                  // chained sweeps: tagged x words + ticket
  luhot::DevBuf scaled_buf;                 // GMRES-IR: block-scaled tiles of the FP32 factor
  luhot::DevBuf oz_buf;                     // FP64 getrf: digit slices of the tensor-core update
  // Look-ahead of the tensor-core LU: a high-priority stream for the panels
  // and the next slab's columns, a low-priority one for the rest of each
  // trailing update, their events (start, ready, rest of even / odd slabs)
  // and the saved move lists of the panels (two slabs x two panels).
  cudaStream_t la_hi = nullptr, la_lo = nullptr;
  cudaEvent_t la_ev[4] = {nullptr, nullptr, nullptr, nullptr};
  luhot::DevBuf la_moves;
  int tc_grid_cap = 0;  // CTAs of the persistent tensor-core update at most (0: one per SM)
  unsigned int chain_epoch = 0;             // tag of the last chained sweep (0 = none)
  double* h_scalars = nullptr;              // pinned: scalars read back by the refinement loop
  void* h_piv = nullptr;                    // pinned pivots staging
  size_t h_piv_bytes = 0;
  int nb_override = 0;
  int fp64_update = LUHOT_UPDATE_AUTO;  // Schur-update engine of fast-mode FP64 getrf
  // The GPU reads pageable host memory through the host's page tables
  // (Grace: address translation services), so large host inputs are copied
  // by SM loads instead of being page-locked for the copy engines.
  bool host_direct = false;
  bool trace = false;  // LUHOT_TRACE=1: refinement steps are reported on stderr
  unsigned long long wait_timeout_ns = 2000000000ull;  // per device-side wait
  std::atomic<int64_t> launches{0};
  // CUDA-event profile (off by default): one event pair per launch.
  bool prof_on = false;
  std::vector<luhot::ProfRecord> prof_records;
  std::vector<cudaEvent_t> prof_event_pool;
  cudaEvent_t prof_pending = nullptr;
};

namespace luhot {

int set_error(luhot_ctx* ctx, int status, const std::string& msg);
int reset_status(luhot_ctx* ctx);
// Synchronises the stream, reads the device status; fills *singular.
int finish_status(luhot_ctx* ctx, int64_t* singular);
int ensure_buf(luhot_ctx* ctx, DevBuf& b, size_t bytes);
// Row-pitched copy on the context's stream: one linear copy when both sides
// are contiguous, a kernel for strided device-to-device, else cudaMemcpy2DAsync.
int copy_2d(luhot_ctx* ctx, void* dst, size_t dpitch, const void* src, size_t spitch, size_t wbytes, size_t rows,
            cudaMemcpyKind kind);

template <typename T>
int getrf_device(luhot_ctx* ctx, int m, int n, T* a, int64_t lda, int* piv, int mode,
                 int64_t* singular);
// One fast-mode FP64 trailing update, a[k.., k..] -= a[k.., 0..k) a[0..k), k..]
// (k <= 64), with the LUHOT_UPDATE_* engine; asynchronous.
int fp64_schur_update(luhot_ctx* ctx, double* a, int64_t lda, int k, int m, int n, int engine);

// Solve with device factors: X (n x nrhs, ldx) <- op(A)^-1 B.  b and x may be
// the same buffer.
// FP32 LU whose Schur updates run on the tensor cores (tcgen05) with
// BF16 / FP16 / TF32 operands (TcKind) and FP32 accumulation; panel width 128.
int getrf_device_tc(luhot_ctx* ctx, int m, int n, float* a, int64_t lda, int* piv, int tc_kind, int64_t* singular);

// The low-precision LU of the mixed-precision solves: FP32 storage and
// panels, Schur updates per LUHOT_PREC_* (FP32 CUDA cores or tcgen05).
int getrf_mixed_device(luhot_ctx* ctx, int m, int n, float* a, int64_t lda, int* piv, int precision,
                       int64_t* singular);

int gesv_ir_device(luhot_ctx* ctx, int n, int nrhs, const double* a, int64_t lda, const double* b, int64_t ldb,
                   double* x, int64_t ldx, int precision, int solver, double tol, int max_iter,
                   luhot_ir_info* info);

// lair's getrf_col_major order (non-standard layouts, exact mode): true when
// the array is not in ndarray's standard layout (lair's dispatch predicate,
// src/lapack/getrf.rs:20-26).  getrf_colmajor_host takes at most 4096 rows
// and returns LUHOT_ERR_UNSUPPORTED beyond.
bool getrf_uses_colmajor(int64_t m, int64_t n, int64_t rs, int64_t cs);
template <typename T>
int getrf_colmajor_host(luhot_ctx* ctx, int64_t m, int64_t n, T* a, int64_t rs, int64_t cs, uint64_t* piv,
                        int64_t* singular);

template <typename T>
int getrs_device(luhot_ctx* ctx, int n, int nrhs, const T* lu, int64_t lda, const int* piv,
                 const T* b, int64_t ldb, T* x, int64_t ldx, int trans, int mode);

// getrs in two parts: compose the interchanges into a permutation once
// (getrs_perm), then apply any number of solves with it (getrs_apply, async;
// w is n x nrhs scratch that must not alias b or x).
int getrs_perm(luhot_ctx* ctx, const int* piv, int n, int* perm);
// Ready flags and ticket of the sync-free triangular sweeps for order n.
int trsv_scratch(luhot_ctx* ctx, int n, int** flags, int** ticket);
// One chained sweep (launch_trsv_chain) on the context's stream with a fresh
// epoch and the context's tagged-word scratch.
template <typename T>
int trsv_chain_sweep(luhot_ctx* ctx, const float* lu, int64_t lda, T* x, int n, bool lower, const T* dinv);
// Inverses of the 128 x 128 diagonal blocks of L and U of an FP32 factor in
// the arithmetic type T (trsv_chain_inverse_elems(n) elements each).
template <typename T>
int chain_invert_blocks(luhot_ctx* ctx, int n, const float* lu, int64_t lda, T* dinv_l, T* dinv_u);
template <typename T>
int getrs_apply(luhot_ctx* ctx, int n, int nrhs, const T* lu, int64_t lda, const int* perm, const T* b,
                int64_t ldb, T* x, int64_t ldx, int trans, int mode, T* w, const T* dinv_l = nullptr,
                const T* dinv_u = nullptr);
// W = the block-scaled off-diagonal tiles of an n x n FP64 factor (see
// launch_scale_blocks), and a single-right-hand-side solve with them:
// x = U^-1 L^-1 P b, b and x strided (x may alias b), v1 and v2 n-vector
// scratch.  Fast mode, untransposed; results agree with getrs_apply to
// fast-mode rounding.
// (TA = float: FP64 tiles of an FP32 factor, for the FP64-arithmetic
// preconditioner of GMRES-IR.)
template <typename TA, typename TW>
int scale_factor_blocks(luhot_ctx* ctx, int n, const TA* lu, int64_t lda, const double* dinv_l, const double* dinv_u,
                        TW* w, int64_t ldw);
// One block-scaled sweep y = T^-1 b (b contiguous, y with stride ldy, y not
// aliasing b) on the context's stream with fresh tagged-word scratch.
template <typename TW>
int scaled_sweep(luhot_ctx* ctx, const TW* w, int64_t ldw, const double* dinv, const double* b, double* y,
                 int64_t ldy, int n, bool lower);
int getrs_scaled_apply(luhot_ctx* ctx, int n, const double* w, int64_t ldw, const int* perm, const double* b,
                       int64_t ldb, double* x, int64_t ldx, const double* dinv_l, const double* dinv_u, double* v1,
                       double* v2);
// Inverses of the diagonal blocks of L (dinv_l) and U (dinv_u) of a
// row-major LU factor; each holds trsv_inverse_elems(n) elements.  They let
// the fast untransposed sweeps of getrs_apply replace each 64-step diagonal
// substitution by a matvec.
template <typename T, typename TA = T>
int invert_diag_blocks(luhot_ctx* ctx, int n, const TA* lu, int64_t lda, T* dinv_l, T* dinv_u);

// Page-locks a caller's host array for the duration of one call (large
// arrays only), so its copies run as DMA at the host link's full rate
// whatever the state of the pageable memory; the stream is synchronised
// before the pages are released.  Ranges this library pinned carry a
// process-wide count of the calls using them (calls on other contexts and
// threads may pass the same array), and a range is unpinned only when its
// last user ends.  Memory the caller registered itself is left alone.
// Strides in elements.
struct HostPin {
  HostPin(luhot_ctx* ctx, const void* base, int64_t m, int64_t n, int64_t rs, int64_t cs, size_t elem);
  ~HostPin();
  HostPin(const HostPin&) = delete;
  HostPin& operator=(const HostPin&) = delete;
  luhot_ctx* ctx = nullptr;
  std::vector<uintptr_t> held;  // start addresses of the pinned ranges this call uses
};

// NVTX range named after the enclosing C entry point (or a phase), shown on
// Nsight Systems / Compute timelines; NVTX is a no-op unless a tool attaches.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};
#define LUHOT_NVTX_FN() ::luhot::NvtxRange luhot_nvtx_fn_(__func__)

// Held by every C entry point: serialises calls on a context, makes its
// device current and clears the last error message.
struct CtxGuard {
  explicit CtxGuard(luhot_ctx* c) : ctx(c), lock(c->mu) {
    cudaSetDevice(c->device);
    ctx->last_error.clear();
  }
  luhot_ctx* ctx;
  std::lock_guard<std::mutex> lock;
};

// Stage a host matrix (any strides) into / out of a row-major device buffer.
template <typename T>
int stage_in(luhot_ctx* ctx, const T* h, int64_t m, int64_t n, int64_t rs, int64_t cs, T* d, int64_t ldd, DevBuf& tmp);
template <typename T>
int stage_out(luhot_ctx* ctx, const T* d, int64_t ldd, T* h, int64_t m, int64_t n, int64_t rs, int64_t cs,
              DevBuf& tmp);
// dst (row-major, ldd) <- transpose of src (rows x cols, lds).
template <typename T>
int launch_transpose(luhot_ctx* ctx, const T* src, int64_t lds, T* dst, int64_t ldd, int rows, int cols);

// Lets launches of `kernel` on the current device request up to the device's
// opt-in shared-memory limit (less the kernel's static shared memory).  The
// attribute is per kernel and device for the whole process, so it is set
// once, under a process-wide lock, and never lowered: a launch on one thread
// can never find the limit lowered by a call on another thread between its
// check and its launch.  Launches still pass their own dynamic size.
cudaError_t allow_max_dynamic_smem(const void* kernel);
template <typename K>
cudaError_t allow_max_dynamic_smem(K* kernel) {
  return allow_max_dynamic_smem(reinterpret_cast<const void*>(kernel));
}

inline void count_launch(luhot_ctx* ctx, int64_t k = 1) { ctx->launches.fetch_add(k); }

// Bracket one kernel launch: prof_begin records a start event on the
// context's stream (when profiling), prof_end the stop event plus the
// launch's algorithmic flops and bytes.  Both count the launch.
void prof_begin(luhot_ctx* ctx, int cls);
void prof_end(luhot_ctx* ctx, int cls, double flops, double bytes);

}  // namespace luhot
