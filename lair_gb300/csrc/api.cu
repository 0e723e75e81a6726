// C ABI of luhot: contexts, host-buffer (drop-in) calls and device calls.
//
// Host matrices arrive with signed element strides (any ndarray view).  They
// are staged into a row-major device buffer (one copy for C order, a copy
// plus an on-device transpose for F order, a host-side pack otherwise), the
// device routine runs, and the result is written back in the caller's own
// layout, as lair's in-place getrf leaves it (src/lapack/getrf.rs:12-27).
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <new>
#include <set>
#include <utility>
#include <vector>

#include "common.cuh"
#include "luhot_internal.h"

namespace luhot {

int set_error(luhot_ctx* ctx, int status, const std::string& msg) {
  if (ctx) ctx->last_error = msg;
  return status;
}

cudaError_t allow_max_dynamic_smem(const void* kernel) {
  static std::mutex mu;
  static std::set<std::pair<const void*, int>> raised;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  if (raised.count({kernel, dev})) return cudaSuccess;
  int optin = 0;
  e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  cudaFuncAttributes fa;
  e = cudaFuncGetAttributes(&fa, kernel);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
  if (e != cudaSuccess) return e;
  raised.insert({kernel, dev});
  return cudaSuccess;
}

int ensure_buf(luhot_ctx* ctx, DevBuf& b, size_t bytes) {
  if (bytes <= b.bytes) return LUHOT_OK;
  if (b.ptr) cudaFree(b.ptr);
  b.ptr = nullptr;
  b.bytes = 0;
  const size_t want = std::max<size_t>(bytes, 256);
  cudaError_t e = cudaMalloc(&b.ptr, want);
  if (e != cudaSuccess) {
    b.ptr = nullptr;
    cudaGetLastError();
    return set_error(ctx, LUHOT_ERR_ALLOC,
                     "device allocation of " + std::to_string(want) + " bytes failed: " + cudaGetErrorString(e));
  }
  b.bytes = want;
  return LUHOT_OK;
}

int reset_status(luhot_ctx* ctx) {
  DeviceStatus init{};
  init.barrier = 0;
  init.error = kDevOk;
  init.singular = -1;
  init.abort = 0;
  init.timeout_where = 0;
  init.timeout_ns = ctx->wait_timeout_ns;
  *ctx->h_status = init;
  LUHOT_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_status, ctx->h_status, sizeof(DeviceStatus),
                                      cudaMemcpyHostToDevice, ctx->stream));
  return LUHOT_OK;
}

int finish_status(luhot_ctx* ctx, int64_t* singular) {
  LUHOT_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->h_status, ctx->d_status, sizeof(DeviceStatus),
                                      cudaMemcpyDeviceToHost, ctx->stream));
  LUHOT_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  const DeviceStatus& s = *ctx->h_status;
  if (s.error == kDevBarrierTimeout)
    return set_error(ctx, LUHOT_ERR_TIMEOUT,
                     "a grid barrier wait timed out at elimination step " + std::to_string(s.timeout_where));
  if (s.error != kDevOk) return set_error(ctx, LUHOT_ERR_CUDA, "device kernel reported an error");
  if (singular) *singular = s.singular;
  return LUHOT_OK;
}

// --------------------------------------------------------------------------
// Layout staging.
// --------------------------------------------------------------------------

// dst (row-major, ldd) <- transpose of src (row-major rows x cols, lds).
template <typename T>
__global__ void transpose_kernel(const T* src, int64_t lds, T* dst, int64_t ldd, int rows, int cols) {
  __shared__ T tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int r = by + j, c = bx + threadIdx.x;
    if (r < rows && c < cols) tile[j][threadIdx.x] = src[(int64_t)r * lds + c];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int r = bx + j, c = by + threadIdx.x;  // dst row = src col
    if (r < cols && c < rows) dst[(int64_t)r * ldd + c] = tile[threadIdx.x][j];
  }
}

template <typename T>
int launch_transpose(luhot_ctx* ctx, const T* src, int64_t lds, T* dst, int64_t ldd, int rows,
                            int cols) {
  dim3 grid((cols + 31) / 32, (rows + 31) / 32), block(32, 8);
  transpose_kernel<T><<<grid, block, 0, ctx->stream>>>(src, lds, dst, ldd, rows, cols);
  count_launch(ctx);
  LUHOT_CUDA_TRY(ctx, cudaGetLastError());
  return LUHOT_OK;
}

static int64_t round_up(int64_t v, int64_t m) { return (v + m - 1) / m * m; }

// Strided device-to-device copy of `rows` rows of `wbytes` bytes (4-byte units).
__global__ void copy_rows_kernel(unsigned char* dst, size_t dpitch, const unsigned char* src, size_t spitch,
                                 size_t words, size_t rows) {
  const size_t total = words * rows;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    const size_t r = t / words, w = t - r * words;
    reinterpret_cast<uint32_t*>(dst + r * dpitch)[w] = reinterpret_cast<const uint32_t*>(src + r * spitch)[w];
  }
}

// Host -> device copy by 16-byte SM loads from pageable host memory that the
// GPU reaches through the host's page tables: no page-locking, and on GB300
// over C2C as fast as the copy engines from locked memory (206 against 189
// GB/s measured for 2 GiB).
__global__ void copy_from_host_kernel(const uint4* __restrict__ src, uint4* __restrict__ dst, size_t n16) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

// A host array of at least this many bytes is copied in by SM loads (on
// hosts whose GPU reads pageable memory) or page-locked for the call.
constexpr size_t kLargeHostBytes = (size_t)8 << 20;

static bool host_direct_source(luhot_ctx* ctx, const void* src, size_t bytes) {
  if (!ctx->host_direct || bytes < kLargeHostBytes || bytes % 16 != 0 ||
      (reinterpret_cast<uintptr_t>(src) & 15) != 0)
    return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, src) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeUnregistered;
}

// A host input (m x n, element strides) that stage_in will copy as one
// contiguous block into a device matrix of leading dimension ldd by SM loads.
static bool direct_input(luhot_ctx* ctx, int64_t m, int64_t n, int64_t rs, int64_t cs, int64_t ldd, size_t elem) {
  if (!ctx->host_direct || m <= 0 || n <= 0 || cs != 1 || (m > 1 && rs != n) || ldd != n) return false;
  return (size_t)(m * n) * elem >= kLargeHostBytes;
}

int copy_2d(luhot_ctx* ctx, void* dst, size_t dpitch, const void* src, size_t spitch, size_t wbytes, size_t rows,
            cudaMemcpyKind kind) {
  if (wbytes == 0 || rows == 0) return LUHOT_OK;
  if ((dpitch == wbytes && spitch == wbytes) || rows == 1) {
    const size_t bytes = wbytes * rows;
    if (kind == cudaMemcpyHostToDevice && (reinterpret_cast<uintptr_t>(dst) & 15) == 0 &&
        host_direct_source(ctx, src, bytes)) {
      copy_from_host_kernel<<<ctx->num_sms * 4, 256, 0, ctx->stream>>>(static_cast<const uint4*>(src),
                                                                     static_cast<uint4*>(dst), bytes / 16);
      count_launch(ctx);
      LUHOT_CUDA_TRY(ctx, cudaGetLastError());
      return LUHOT_OK;
    }
    LUHOT_CUDA_TRY(ctx, cudaMemcpyAsync(dst, src, bytes, kind, ctx->stream));
    return LUHOT_OK;
  }
  if (kind == cudaMemcpyDeviceToDevice && wbytes % 4 == 0 && dpitch % 4 == 0 && spitch % 4 == 0 &&
      (reinterpret_cast<uintptr_t>(dst) & 3) == 0 && (reinterpret_cast<uintptr_t>(src) & 3) == 0) {
    const size_t total = wbytes / 4 * rows;
    const int blocks = (int)std::min<size_t>((total + 255) / 256, (size_t)ctx->num_sms * 8);
    copy_rows_kernel<<<blocks, 256, 0, ctx->stream>>>(static_cast<unsigned char*>(dst), dpitch,
                                                      static_cast<const unsigned char*>(src), spitch, wbytes / 4, rows);
    count_launch(ctx);
    LUHOT_CUDA_TRY(ctx, cudaGetLastError());
    return LUHOT_OK;
  }
  LUHOT_CUDA_TRY(ctx, cudaMemcpy2DAsync(dst, dpitch, src, spitch, wbytes, rows, kind, ctx->stream));
  return LUHOT_OK;
}

// Two co-resident CTAs wait for three arrivals: the wait can only end by its
// time limit.  Exercises the timeout path of grid_barrier without a fault.
__global__ void unreachable_barrier_kernel(DeviceStatus* st) {
  grid_barrier(st, gridDim.x + 1, 0xFFFFull);
}

static int launch_unreachable_barrier(luhot_ctx* ctx) {
  void* args[] = {&ctx->d_status};
  LUHOT_CUDA_TRY(ctx, cudaLaunchCooperativeKernel((void*)unreachable_barrier_kernel, dim3(2), dim3(32),
                                                  args, 0, ctx->stream));
  count_launch(ctx);
  return LUHOT_OK;
}

enum class Layout { kC, kF, kOther };

// kC: rows contiguous with a positive pitch >= n (one 2-D copy);
// kF: columns contiguous with a positive pitch >= m (copy + transpose);
// kOther: anything else, e.g. negative strides (packed on the host).
static Layout classify(int64_t m, int64_t n, int64_t rs, int64_t cs) {
  if ((n <= 1 || cs == 1) && (m <= 1 || rs >= std::max<int64_t>(n, 1))) return Layout::kC;
  if ((m <= 1 || rs == 1) && (n <= 1 || cs >= std::max<int64_t>(m, 1))) return Layout::kF;
  return Layout::kOther;
}

// Host (m x n, rs, cs) -> device row-major (ldd).  `tmp` is device scratch
// of at least m*n elements for the F-order path.
template <typename T>
int stage_in(luhot_ctx* ctx, const T* h, int64_t m, int64_t n, int64_t rs, int64_t cs, T* d,
                    int64_t ldd, DevBuf& tmp) {
  if (m == 0 || n == 0) return LUHOT_OK;
  const Layout lay = classify(m, n, rs, cs);
  if (lay == Layout::kC) {
    const int64_t src_ld = (m <= 1) ? n : rs;
    {
      int rc_ = copy_2d(ctx, d, ldd * sizeof(T), h, src_ld * sizeof(T), n * sizeof(T), m,
                                          cudaMemcpyHostToDevice);
      if (rc_) return rc_;
    }
    return LUHOT_OK;
  }
  if (lay == Layout::kF) {
    const int64_t src_ld = (n <= 1) ? m : cs;
    int rc = ensure_buf(ctx, tmp, (size_t)m * n * sizeof(T));
    if (rc) return rc;
    T* t = static_cast<T*>(tmp.ptr);  // n x m row-major (= A^T)
    {
      int rc_ = copy_2d(ctx, t, m * sizeof(T), h, src_ld * sizeof(T), m * sizeof(T), n,
                                          cudaMemcpyHostToDevice);
      if (rc_) return rc_;
    }
    return launch_transpose<T>(ctx, t, m, d, ldd, (int)n, (int)m);
  }
  std::vector<T> packed((size_t)m * n);
  for (int64_t i = 0; i < m; ++i)
    for (int64_t j = 0; j < n; ++j) packed[(size_t)i * n + j] = h[i * rs + j * cs];
  {
      int rc_ = copy_2d(ctx, d, ldd * sizeof(T), packed.data(), n * sizeof(T), n * sizeof(T), m,
                                        cudaMemcpyHostToDevice);
      if (rc_) return rc_;
    }
  LUHOT_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));  // packed goes out of scope
  return LUHOT_OK;
}

// Device row-major (ldd) -> host (m x n, rs, cs).  Synchronises the stream.
template <typename T>
int stage_out(luhot_ctx* ctx, const T* d, int64_t ldd, T* h, int64_t m, int64_t n, int64_t rs,
                     int64_t cs, DevBuf& tmp) {
  if (m == 0 || n == 0) return LUHOT_OK;
  const Layout lay = classify(m, n, rs, cs);
  if (lay == Layout::kC) {
    const int64_t dst_ld = (m <= 1) ? n : rs;
    {
      int rc_ = copy_2d(ctx, h, dst_ld * sizeof(T), d, ldd * sizeof(T), n * sizeof(T), m,
                                          cudaMemcpyDeviceToHost);
      if (rc_) return rc_;
    }
    LUHOT_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return LUHOT_OK;
  }
  if (lay == Layout::kF) {
    const int64_t dst_ld = (n <= 1) ? m : cs;
    int rc = ensure_buf(ctx, tmp, (size_t)m * n * sizeof(T));
    if (rc) return rc;
    T* t = static_cast<T*>(tmp.ptr);
    rc = launch_transpose<T>(ctx, d, ldd, t, m, (int)m, (int)n);
    if (rc) return rc;
    {
      int rc_ = copy_2d(ctx, h, dst_ld * sizeof(T), t, m * sizeof(T), m * sizeof(T), n,
                                          cudaMemcpyDeviceToHost);
      if (rc_) return rc_;
    }
    LUHOT_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return LUHOT_OK;
  }
  std::vector<T> packed((size_t)m * n);
  {
      int rc_ = copy_2d(ctx, packed.data(), n * sizeof(T), d, ldd * sizeof(T), n * sizeof(T), m,
                                        cudaMemcpyDeviceToHost);
      if (rc_) return rc_;
    }
  LUHOT_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  for (int64_t i = 0; i < m; ++i)
    for (int64_t j = 0; j < n; ++j) h[i * rs + j * cs] = packed[(size_t)i * n + j];
  return LUHOT_OK;
}

template int stage_in<double>(luhot_ctx*, const double*, int64_t, int64_t, int64_t, int64_t, double*, int64_t,
                              DevBuf&);
template int stage_in<float>(luhot_ctx*, const float*, int64_t, int64_t, int64_t, int64_t, float*, int64_t, DevBuf&);
template int stage_out<double>(luhot_ctx*, const double*, int64_t, double*, int64_t, int64_t, int64_t, int64_t,
                               DevBuf&);
template int stage_out<float>(luhot_ctx*, const float*, int64_t, float*, int64_t, int64_t, int64_t, int64_t, DevBuf&);
template int launch_transpose<double>(luhot_ctx*, const double*, int64_t, double*, int64_t, int, int);

namespace {
// Host ranges this library page-locked, keyed by start address, with the
// number of calls currently using each.  cudaHostRegister refuses
// overlapping ranges, so the ranges are disjoint.
struct PinnedRange {
  uintptr_t end;
  int users;
};
std::mutex g_pin_mu;
std::map<uintptr_t, PinnedRange> g_pinned;
}  // namespace

HostPin::HostPin(luhot_ctx* c, const void* base, int64_t m, int64_t n, int64_t rs, int64_t cs, size_t elem)
    : ctx(c) {
  if (!base || m <= 0 || n <= 0 || rs < 0 || cs < 0) return;
  const size_t span = ((size_t)(m - 1) * (size_t)rs + (size_t)(n - 1) * (size_t)cs + 1) * elem;
  if (span < kLargeHostBytes) return;
  const uintptr_t lo = reinterpret_cast<uintptr_t>(base), hi = lo + span;
  std::lock_guard<std::mutex> lock(g_pin_mu);
  // A call on another context may have pinned this array (or part of it):
  // hold those ranges for this call instead of registering again, so that
  // the other call's release cannot unpin them under this call's copies.
  auto it = g_pinned.upper_bound(lo);
  if (it != g_pinned.begin()) --it;
  for (; it != g_pinned.end() && it->first < hi; ++it) {
    if (it->second.end > lo) {
      ++it->second.users;
      held.push_back(it->first);
    }
  }
  if (!held.empty()) return;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, base) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  if (at.type != cudaMemoryTypeUnregistered) return;  // the caller's own pinned or managed memory
  if (cudaHostRegister(const_cast<void*>(base), span, cudaHostRegisterDefault) == cudaSuccess) {
    g_pinned[lo] = PinnedRange{hi, 1};
    held.push_back(lo);
  } else {
    cudaGetLastError();
  }
}

HostPin::~HostPin() {
  if (held.empty()) return;
  cudaStreamSynchronize(ctx->stream);  // this call's copies from the range are done
  std::lock_guard<std::mutex> lock(g_pin_mu);
  for (uintptr_t key : held) {
    auto it = g_pinned.find(key);
    if (it == g_pinned.end()) continue;
    if (--it->second.users == 0) {
      cudaHostUnregister(reinterpret_cast<void*>(key));
      cudaGetLastError();
      g_pinned.erase(it);
    }
  }
}

// ndarray 0.17's ArrayBase::is_contiguous for two axes: the elements fill
// one block of memory in C or F order, strides of either sign (axes of
// length 1 take any stride).  lair's equation::solve copies A with to_owned
// (src/equation.rs:54), which keeps the strides of such an array and makes
// any other array standard.
static bool ndarray_contiguous(int64_t m, int64_t n, int64_t rs, int64_t cs) {
  if (m == 0 || n == 0) return true;
  const int64_t ars = rs < 0 ? -rs : rs, acs = cs < 0 ? -cs : cs;
  if (m == 1) return n == 1 || acs == 1;
  if (n == 1) return ars == 1;
  return (acs == 1 && ars == n) || (ars == 1 && acs == m);
}

static bool dims_ok(int64_t m, int64_t n) {
  return m >= 0 && n >= 0 && m < (int64_t)INT32_MAX && n < (int64_t)INT32_MAX &&
         (m == 0 || n == 0 || m * n / n == m);
}

// Padded leading dimension for device copies (whole 256-byte rows).
template <typename T>
static int64_t dev_ld(int64_t n) {
  return round_up(std::max<int64_t>(n, 1), 256 / (int64_t)sizeof(T));
}

template <typename T>
static int getrf_host(luhot_ctx* ctx, int64_t m, int64_t n, T* a, int64_t rs, int64_t cs, uint64_t* piv,
                      int64_t* singular, int mode) {
  if (!dims_ok(m, n)) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "getrf: invalid dimensions");
  if (mode != LUHOT_MODE_FAST && mode != LUHOT_MODE_EXACT)
    return set_error(ctx, LUHOT_ERR_INVALID_ARG, "getrf: unknown mode");
  const int64_t k = std::min(m, n);
  if ((m * n > 0 && !a) || (k > 0 && !piv))
    return set_error(ctx, LUHOT_ERR_INVALID_ARG, "getrf: null pointer");
  if (singular) *singular = -1;
  if (k == 0) return LUHOT_OK;
  // lair factors non-standard layouts with its column-major (Crout) order
  // (src/lapack/getrf.rs:22-26); exact mode follows it bit for bit.
  if (mode == LUHOT_MODE_EXACT && getrf_uses_colmajor(m, n, rs, cs))
    return getrf_colmajor_host<T>(ctx, m, n, a, rs, cs, piv, singular);
  const int64_t lda = dev_ld<T>(n);
  HostPin pin_a(ctx, a, m, n, rs, cs, sizeof(T));
  int rc = ensure_buf(ctx, ctx->work[0], (size_t)m * lda * sizeof(T));
  if (rc) return rc;
  rc = ensure_buf(ctx, ctx->piv_buf, (size_t)k * sizeof(int));
  if (rc) return rc;
  T* d_a = static_cast<T*>(ctx->work[0].ptr);
  int* d_piv = static_cast<int*>(ctx->piv_buf.ptr);
  rc = stage_in<T>(ctx, a, m, n, rs, cs, d_a, lda, ctx->work[1]);
  if (rc) return rc;
  int64_t sing = -1;
  rc = getrf_device<T>(ctx, (int)m, (int)n, d_a, lda, d_piv, mode, &sing);
  if (rc) return rc;
  rc = stage_out<T>(ctx, d_a, lda, a, m, n, rs, cs, ctx->work[1]);
  if (rc) return rc;
  std::vector<int> hp((size_t)k);
  LUHOT_CUDA_TRY(ctx, cudaMemcpy(hp.data(), d_piv, (size_t)k * sizeof(int), cudaMemcpyDeviceToHost));
  for (int64_t i = 0; i < k; ++i) piv[i] = (uint64_t)hp[(size_t)i];
  if (singular) *singular = sing;
  return LUHOT_OK;
}

template <typename T>
static int getrs_host(luhot_ctx* ctx, int64_t n, int64_t nrhs, const T* lu, int64_t lu_rs, int64_t lu_cs,
                      const uint64_t* piv, const T* b, int64_t b_rs, int64_t b_cs, T* x, int64_t x_rs,
                      int64_t x_cs, int trans, int mode) {
  if (!dims_ok(n, nrhs)) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "getrs: invalid dimensions");
  if (mode != LUHOT_MODE_FAST && mode != LUHOT_MODE_EXACT)
    return set_error(ctx, LUHOT_ERR_INVALID_ARG, "getrs: unknown mode");
  if (n == 0 || nrhs == 0) return LUHOT_OK;
  if (!lu || !piv || !b || !x) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "getrs: null pointer");
  for (int64_t i = 0; i < n; ++i)
    if (piv[i] >= (uint64_t)n)
      return set_error(ctx, LUHOT_ERR_INVALID_ARG, "getrs: pivot index out of range");
  const int64_t lda = dev_ld<T>(n);
  const int64_t ldb = nrhs;
  HostPin pin_lu(ctx, lu, n, n, lu_rs, lu_cs, sizeof(T));
  int rc = ensure_buf(ctx, ctx->work[0], (size_t)n * lda * sizeof(T));
  if (rc) return rc;
  rc = ensure_buf(ctx, ctx->work[2], (size_t)n * ldb * sizeof(T));
  if (rc) return rc;
  rc = ensure_buf(ctx, ctx->piv_buf, (size_t)n * sizeof(int));
  if (rc) return rc;
  T* d_lu = static_cast<T*>(ctx->work[0].ptr);
  T* d_b = static_cast<T*>(ctx->work[2].ptr);
  int* d_piv = static_cast<int*>(ctx->piv_buf.ptr);
  rc = stage_in<T>(ctx, lu, n, n, lu_rs, lu_cs, d_lu, lda, ctx->work[1]);
  if (rc) return rc;
  rc = stage_in<T>(ctx, b, n, nrhs, b_rs, b_cs, d_b, ldb, ctx->work[1]);
  if (rc) return rc;
  std::vector<int> hp((size_t)n);
  for (int64_t i = 0; i < n; ++i) hp[(size_t)i] = (int)piv[i];
  LUHOT_CUDA_TRY(ctx, cudaMemcpyAsync(d_piv, hp.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice,
                                      ctx->stream));
  rc = getrs_device<T>(ctx, (int)n, (int)nrhs, d_lu, lda, d_piv, d_b, ldb, d_b, ldb, trans, mode);
  if (rc) return rc;
  rc = stage_out<T>(ctx, d_b, ldb, x, n, nrhs, x_rs, x_cs, ctx->work[1]);
  if (rc) return rc;
  return LUHOT_OK;
}

}  // namespace luhot

using namespace luhot;

namespace {
using Guard = luhot::CtxGuard;
}  // namespace

extern "C" {

const char* luhot_version(void) { return "0.1.0"; }

const char* luhot_status_string(int status) {
  switch (status) {
    case LUHOT_OK: return "ok";
    case LUHOT_ERR_INVALID_ARG: return "invalid argument";
    case LUHOT_ERR_CUDA: return "CUDA error";
    case LUHOT_ERR_ALLOC: return "allocation failed";
    case LUHOT_ERR_TIMEOUT: return "device wait timed out";
    case LUHOT_ERR_NOT_CONVERGED: return "iterative refinement did not converge";
    case LUHOT_ERR_SINGULAR: return "matrix is singular";
    case LUHOT_ERR_UNSUPPORTED: return "unsupported size or option";
    default: return "unknown status";
  }
}

int luhot_create(luhot_ctx** out, int device) {
  if (!out) return LUHOT_ERR_INVALID_ARG;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return LUHOT_ERR_CUDA;
  }
  if (device < 0 || device >= count) return LUHOT_ERR_INVALID_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return LUHOT_ERR_CUDA;
  luhot_ctx* ctx = new (std::nothrow) luhot_ctx();
  if (!ctx) return LUHOT_ERR_ALLOC;
  ctx->device = device;
  {
    const char* tr = std::getenv("LUHOT_TRACE");
    ctx->trace = tr && tr[0] == '1';
  }
  cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  cudaDeviceGetAttribute(&ctx->max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  {
    int pageable = 0, host_tables = 0;
    cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device);
    cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device);
    ctx->host_direct = pageable == 1 && host_tables == 1;
    cudaGetLastError();
  }
  bool ok = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) == cudaSuccess;
  ctx->stream = ctx->own_stream;
  ok = ok && cudaMalloc(&ctx->d_status, sizeof(DeviceStatus)) == cudaSuccess;
  ok = ok && cudaMallocHost(&ctx->h_status, sizeof(DeviceStatus)) == cudaSuccess;
  ok = ok && cudaMallocHost(&ctx->h_scalars, kIrScalarSlots * sizeof(double)) == cudaSuccess;
  ok = ok && cudaMalloc(&ctx->panel_scratch, kPanelScratchBytes) == cudaSuccess;
  if (!ok || ctx->num_sms > kMaxPanelCtas) {
    cudaGetLastError();
    luhot_destroy(ctx);
    return LUHOT_ERR_CUDA;
  }
  *out = ctx;
  return LUHOT_OK;
}

void luhot_destroy(luhot_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->own_stream) cudaStreamSynchronize(ctx->own_stream);
  for (auto& b : ctx->work)
    if (b.ptr) cudaFree(b.ptr);
  if (ctx->piv_buf.ptr) cudaFree(ctx->piv_buf.ptr);
  if (ctx->perm_buf.ptr) cudaFree(ctx->perm_buf.ptr);
  if (ctx->trsv_buf.ptr) cudaFree(ctx->trsv_buf.ptr);
  if (ctx->panel_scratch) cudaFree(ctx->panel_scratch);
  if (ctx->d_status) cudaFree(ctx->d_status);
  if (ctx->h_status) cudaFreeHost(ctx->h_status);
  if (ctx->h_scalars) cudaFreeHost(ctx->h_scalars);
  for (auto& b : ctx->ir_buf)
    if (b.ptr) cudaFree(b.ptr);
  if (ctx->adj_buf.ptr) cudaFree(ctx->adj_buf.ptr);
  if (ctx->tc_buf.ptr) cudaFree(ctx->tc_buf.ptr);
  if (ctx->dinv_buf.ptr) cudaFree(ctx->dinv_buf.ptr);
  if (ctx->chain_buf.ptr) cudaFree(ctx->chain_buf.ptr);
  if (ctx->scaled_buf.ptr) cudaFree(ctx->scaled_buf.ptr);
  if (ctx->oz_buf.ptr) cudaFree(ctx->oz_buf.ptr);
  if (ctx->la_moves.ptr) cudaFree(ctx->la_moves.ptr);
  for (auto& e : ctx->la_ev)
    if (e) cudaEventDestroy(e);
  if (ctx->la_hi) cudaStreamDestroy(ctx->la_hi);
  if (ctx->la_lo) cudaStreamDestroy(ctx->la_lo);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
}

const char* luhot_last_error(const luhot_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

int luhot_set_stream(luhot_ctx* ctx, void* cuda_stream) {
  if (!ctx) return LUHOT_ERR_INVALID_ARG;
  Guard g(ctx);
  ctx->stream = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : ctx->own_stream;
  return LUHOT_OK;
}

int luhot_set_block(luhot_ctx* ctx, int nb) {
  if (!ctx || nb < 0 || nb > kDefaultPanelWidth) return LUHOT_ERR_INVALID_ARG;
  Guard g(ctx);
  ctx->nb_override = nb;
  return LUHOT_OK;
}

int luhot_set_fp64_update(luhot_ctx* ctx, int engine) {
  if (!ctx || engine < LUHOT_UPDATE_AUTO || engine > LUHOT_UPDATE_OZAKI) return LUHOT_ERR_INVALID_ARG;
  Guard g(ctx);
  ctx->fp64_update = engine;
  return LUHOT_OK;
}

int luhot_dschur_update_dev(luhot_ctx* ctx, int64_t m, int64_t n, int64_t k, double* d_a, int64_t lda, int engine) {
  LUHOT_NVTX_FN();
  if (!ctx) return LUHOT_ERR_INVALID_ARG;
  Guard g(ctx);
  if (!dims_ok(m, n) || k < 1 || k > kDefaultPanelWidth || k > std::min(m, n) || lda < std::max<int64_t>(1, n))
    return set_error(ctx, LUHOT_ERR_INVALID_ARG, "schur update: invalid dimensions");
  if (engine < LUHOT_UPDATE_AUTO || engine > LUHOT_UPDATE_OZAKI)
    return set_error(ctx, LUHOT_ERR_INVALID_ARG, "schur update: unknown engine");
  if (!d_a) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "schur update: null pointer");
  int rc = reset_status(ctx);
  if (rc) return rc;
  rc = fp64_schur_update(ctx, d_a, lda, (int)k, (int)m, (int)n, engine);
  if (rc) return rc;
  return finish_status(ctx, nullptr);
}

int64_t luhot_launch_count(const luhot_ctx* ctx) { return ctx ? ctx->launches.load() : 0; }

int luhot_selftest_wait_timeout(luhot_ctx* ctx, int64_t timeout_ms) {
  if (!ctx || timeout_ms <= 0 || timeout_ms > 10000) return LUHOT_ERR_INVALID_ARG;
  Guard g(ctx);
  const unsigned long long saved = ctx->wait_timeout_ns;
  ctx->wait_timeout_ns = (unsigned long long)timeout_ms * 1000000ull;
  int rc = reset_status(ctx);
  ctx->wait_timeout_ns = saved;
  if (rc) return rc;
  rc = launch_unreachable_barrier(ctx);
  if (rc) return rc;
  return finish_status(ctx, nullptr);
}

int luhot_dgetrf(luhot_ctx* ctx, int64_t m, int64_t n, double* a, int64_t rs, int64_t cs, uint64_t* piv,
                 int64_t* singular, int mode) {
  LUHOT_NVTX_FN();
  if (!ctx) return LUHOT_ERR_INVALID_ARG;
  Guard g(ctx);
  return getrf_host<double>(ctx, m, n, a, rs, cs, piv, singular, mode);
}

int luhot_sgetrf(luhot_ctx* ctx, int64_t m, int64_t n, float* a, int64_t rs, int64_t cs, uint64_t* piv,
                 int64_t* singular, int mode) {
  LUHOT_NVTX_FN();
  if (!ctx) return LUHOT_ERR_INVALID_ARG;
  Guard g(ctx);
  return getrf_host<float>(ctx, m, n, a, rs, cs, piv, singular, mode);
}

int luhot_dgetrs(luhot_ctx* ctx, int64_t n, int64_t nrhs, const double* lu, int64_t lu_rs, int64_t lu_cs,
                 const uint64_t* piv, const double* b, int64_t b_rs, int64_t b_cs, double* x, int64_t x_rs,
                 int64_t x_cs, int trans, int mode) {
  LUHOT_NVTX_FN();
  if (!ctx) return LUHOT_ERR_INVALID_ARG;
  Guard g(ctx);
  return getrs_host<double>(ctx, n, nrhs, lu, lu_rs, lu_cs, piv, b, b_rs, b_cs, x, x_rs, x_cs, trans, mode);
}

int luhot_sgetrs(luhot_ctx* ctx, int64_t n, int64_t nrhs, const float* lu, int64_t lu_rs, int64_t lu_cs,
                 const uint64_t* piv, const float* b, int64_t b_rs, int64_t b_cs, float* x, int64_t x_rs,
                 int64_t x_cs, int trans, int mode) {
  LUHOT_NVTX_FN();
  if (!ctx) return LUHOT_ERR_INVALID_ARG;
  Guard g(ctx);
  return getrs_host<float>(ctx, n, nrhs, lu, lu_rs, lu_cs, piv, b, b_rs, b_cs, x, x_rs, x_cs, trans, mode);
}

int luhot_dgesv(luhot_ctx* ctx, int64_t n, int64_t nrhs, const double* a, int64_t rs, int64_t cs,
                const double* b, int64_t b_rs, int64_t b_cs, double* x, int64_t x_rs, int64_t x_cs, int mode) {
  LUHOT_NVTX_FN();
  if (!ctx) return LUHOT_ERR_INVALID_ARG;
  Guard g(ctx);
  if (!dims_ok(n, nrhs) || !dims_ok(n, n)) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "gesv: invalid dimensions");
  if (mode != LUHOT_MODE_FAST && mode != LUHOT_MODE_EXACT)
    return set_error(ctx, LUHOT_ERR_INVALID_ARG, "gesv: unknown mode");
  if (n == 0 || nrhs == 0) return LUHOT_OK;
  if (!a || !b || !x) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "gesv: null pointer");
  const int64_t lda = dev_ld<double>(n);
  // A and B are only read: on hosts whose GPU reads pageable memory their
  // contiguous row-major copies go by SM loads (copy_2d) with no page-locking.
  HostPin pin_a(ctx, direct_input(ctx, n, n, rs, cs, lda, sizeof(double)) ? nullptr : a, n, n, rs, cs, sizeof(double));
  HostPin pin_b(ctx, direct_input(ctx, n, nrhs, b_rs, b_cs, nrhs, sizeof(double)) ? nullptr : b, n, nrhs, b_rs, b_cs,
                sizeof(double));
  HostPin pin_x(ctx, x, n, nrhs, x_rs, x_cs, sizeof(double));
  int rc = ensure_buf(ctx, ctx->work[0], (size_t)n * lda * sizeof(double));
  if (rc) return rc;
  rc = ensure_buf(ctx, ctx->work[2], (size_t)n * nrhs * sizeof(double));
  if (rc) return rc;
  rc = ensure_buf(ctx, ctx->piv_buf, (size_t)n * sizeof(int));
  if (rc) return rc;
  double* d_a = static_cast<double*>(ctx->work[0].ptr);
  double* d_b = static_cast<double*>(ctx->work[2].ptr);
  int* d_piv = static_cast<int*>(ctx->piv_buf.ptr);
  int64_t sing = -1;
  if (mode == LUHOT_MODE_EXACT && getrf_uses_colmajor(n, n, rs, cs) && ndarray_contiguous(n, n, rs, cs)) {
    // lair's copy of a contiguous non-standard array keeps its layout, so
    // getrf factors it in the column-major order (src/lapack/getrf.rs:20-26).
    std::vector<double> colmajor((size_t)n * n);
    for (int64_t j = 0; j < n; ++j)
      for (int64_t i = 0; i < n; ++i) colmajor[(size_t)j * n + i] = a[i * rs + j * cs];
    std::vector<uint64_t> hpiv((size_t)n);
    rc = getrf_colmajor_host<double>(ctx, n, n, colmajor.data(), 1, n, hpiv.data(), &sing);
    if (rc) return rc;
    if (sing >= 0) return set_error(ctx, LUHOT_ERR_SINGULAR, "`a` is a singular matrix");
    rc = stage_in<double>(ctx, colmajor.data(), n, n, 1, n, d_a, lda, ctx->work[1]);
    if (rc) return rc;
    std::vector<int> hp((size_t)n);
    for (int64_t i = 0; i < n; ++i) hp[(size_t)i] = (int)hpiv[(size_t)i];
    LUHOT_CUDA_TRY(ctx, cudaMemcpyAsync(d_piv, hp.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice,
                                        ctx->stream));
    LUHOT_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));  // colmajor and hp go out of scope
    rc = stage_in<double>(ctx, b, n, nrhs, b_rs, b_cs, d_b, nrhs, ctx->work[1]);
    if (rc) return rc;
    rc = getrs_device<double>(ctx, (int)n, (int)nrhs, d_a, lda, d_piv, d_b, nrhs, d_b, nrhs, 0, mode);
    if (rc) return rc;
    return stage_out<double>(ctx, d_b, nrhs, x, n, nrhs, x_rs, x_cs, ctx->work[1]);
  }
  rc = stage_in<double>(ctx, a, n, n, rs, cs, d_a, lda, ctx->work[1]);
  if (rc) return rc;
  rc = stage_in<double>(ctx, b, n, nrhs, b_rs, b_cs, d_b, nrhs, ctx->work[1]);
  if (rc) return rc;
  rc = getrf_device<double>(ctx, (int)n, (int)n, d_a, lda, d_piv, mode, &sing);
  if (rc) return rc;
  if (sing >= 0) return set_error(ctx, LUHOT_ERR_SINGULAR, "`a` is a singular matrix");
  rc = getrs_device<double>(ctx, (int)n, (int)nrhs, d_a, lda, d_piv, d_b, nrhs, d_b, nrhs, 0, mode);
  if (rc) return rc;
  return stage_out<double>(ctx, d_b, nrhs, x, n, nrhs, x_rs, x_cs, ctx->work[1]);
}

int luhot_dgetrf_dev(luhot_ctx* ctx, int64_t m, int64_t n, double* d_a, int64_t lda, int32_t* d_piv,
                     int64_t* singular, int mode) {
  LUHOT_NVTX_FN();
  if (!ctx) return LUHOT_ERR_INVALID_ARG;
  Guard g(ctx);
  if (!dims_ok(m, n)) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "getrf: invalid dimensions");
  if (std::min(m, n) > 0 && (!d_a || !d_piv)) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "getrf: null pointer");
  return getrf_device<double>(ctx, (int)m, (int)n, d_a, lda, d_piv, mode, singular);
}

int luhot_sgetrf_dev(luhot_ctx* ctx, int64_t m, int64_t n, float* d_a, int64_t lda, int32_t* d_piv,
                     int64_t* singular, int mode) {
  LUHOT_NVTX_FN();
  if (!ctx) return LUHOT_ERR_INVALID_ARG;
  Guard g(ctx);
  if (!dims_ok(m, n)) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "getrf: invalid dimensions");
  if (std::min(m, n) > 0 && (!d_a || !d_piv)) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "getrf: null pointer");
  return getrf_device<float>(ctx, (int)m, (int)n, d_a, lda, d_piv, mode, singular);
}

int luhot_sgetrf_mixed_dev(luhot_ctx* ctx, int64_t m, int64_t n, float* d_a, int64_t lda, int32_t* d_piv,
                           int precision, int64_t* singular) {
  LUHOT_NVTX_FN();
  if (!ctx) return LUHOT_ERR_INVALID_ARG;
  Guard g(ctx);
  if (!dims_ok(m, n)) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "getrf: invalid dimensions");
  if (std::min(m, n) > 0 && (!d_a || !d_piv)) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "getrf: null pointer");
  return getrf_mixed_device(ctx, (int)m, (int)n, d_a, lda, d_piv, precision, singular);
}

int luhot_dgetrs_dev(luhot_ctx* ctx, int64_t n, int64_t nrhs, const double* d_lu, int64_t lda,
                     const int32_t* d_piv, double* d_b, int64_t ldb, int trans, int mode) {
  LUHOT_NVTX_FN();
  if (!ctx) return LUHOT_ERR_INVALID_ARG;
  Guard g(ctx);
  if (!dims_ok(n, nrhs)) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "getrs: invalid dimensions");
  if (n > 0 && nrhs > 0 && (!d_lu || !d_piv || !d_b)) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "getrs: null pointer");
  return getrs_device<double>(ctx, (int)n, (int)nrhs, d_lu, lda, d_piv, d_b, ldb, d_b, ldb, trans, mode);
}

int luhot_sgetrs_dev(luhot_ctx* ctx, int64_t n, int64_t nrhs, const float* d_lu, int64_t lda,
                     const int32_t* d_piv, float* d_b, int64_t ldb, int trans, int mode) {
  LUHOT_NVTX_FN();
  if (!ctx) return LUHOT_ERR_INVALID_ARG;
  Guard g(ctx);
  if (!dims_ok(n, nrhs)) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "getrs: invalid dimensions");
  if (n > 0 && nrhs > 0 && (!d_lu || !d_piv || !d_b)) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "getrs: null pointer");
  return getrs_device<float>(ctx, (int)n, (int)nrhs, d_lu, lda, d_piv, d_b, ldb, d_b, ldb, trans, mode);
}

int luhot_dgesv_ir_dev(luhot_ctx* ctx, int64_t n, int64_t nrhs, const double* d_a, int64_t lda,
                       const double* d_b, int64_t ldb, double* d_x, int64_t ldx, int precision, int solver,
                       double tol, int max_iter, luhot_ir_info* info) {
  LUHOT_NVTX_FN();
  if (!ctx || !info) return LUHOT_ERR_INVALID_ARG;
  Guard g(ctx);
  if (!dims_ok(n, nrhs) || !dims_ok(n, n)) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "gesv_ir: invalid dimensions");
  if (n > 0 && nrhs > 0 && (!d_a || !d_b || !d_x)) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "gesv_ir: null pointer");
  return gesv_ir_device(ctx, (int)n, (int)nrhs, d_a, lda, d_b, ldb, d_x, ldx, precision, solver, tol, max_iter, info);
}

int luhot_dgesv_ir(luhot_ctx* ctx, int64_t n, int64_t nrhs, const double* a, int64_t rs, int64_t cs,
                   const double* b, int64_t b_rs, int64_t b_cs, double* x, int64_t x_rs, int64_t x_cs, int precision,
                   int solver, double tol, int max_iter, luhot_ir_info* info) {
  LUHOT_NVTX_FN();
  if (!ctx || !info) return LUHOT_ERR_INVALID_ARG;
  Guard g(ctx);
  if (!dims_ok(n, nrhs) || !dims_ok(n, n)) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "gesv_ir: invalid dimensions");
  if (n == 0 || nrhs == 0) {
    *info = luhot_ir_info{};
    info->converged = 1;
    info->singular = -1;
    return LUHOT_OK;
  }
  if (!a || !b || !x) return set_error(ctx, LUHOT_ERR_INVALID_ARG, "gesv_ir: null pointer");
  const int64_t lda = dev_ld<double>(n);
  int rc = ensure_buf(ctx, ctx->work[0], (size_t)n * lda * sizeof(double));
  if (rc) return rc;
  rc = ensure_buf(ctx, ctx->work[2], (size_t)n * nrhs * 2 * sizeof(double));
  if (rc) return rc;
  double* d_a = static_cast<double*>(ctx->work[0].ptr);
  double* d_b = static_cast<double*>(ctx->work[2].ptr);
  double* d_x = d_b + (size_t)n * nrhs;
  rc = stage_in<double>(ctx, a, n, n, rs, cs, d_a, lda, ctx->work[1]);
  if (rc) return rc;
  rc = stage_in<double>(ctx, b, n, nrhs, b_rs, b_cs, d_b, nrhs, ctx->work[1]);
  if (rc) return rc;
  rc = gesv_ir_device(ctx, (int)n, (int)nrhs, d_a, lda, d_b, nrhs, d_x, nrhs, precision, solver, tol, max_iter, info);
  if (rc != LUHOT_OK && rc != LUHOT_ERR_NOT_CONVERGED) return rc;
  const std::string msg = ctx->last_error;
  const int rc2 = stage_out<double>(ctx, d_x, nrhs, x, n, nrhs, x_rs, x_cs, ctx->work[1]);
  if (rc2) return rc2;
  if (rc) ctx->last_error = msg;
  return rc;
}

}  // extern "C"
