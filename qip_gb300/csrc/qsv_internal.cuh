// Internal declarations shared by the translation units of libqsv.so.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>

#include "../../include/qsv.h"

// Largest number of qubit positions a single call may name (targets + controls).
constexpr int QSV_MAXQ = 40;
// Largest register width of a state handle (2^34 complex64 = 128 GiB).
constexpr int QSV_MAXN = 34;
constexpr int QSV_THREADS = 256;

struct qsv_state {
  int n = 0;
  int dtype = QSV_C64;
  int device = 0;
  int sm_count = 0;
  size_t amp_bytes = 8;
  void* d_amp = nullptr;
  cudaStream_t stream = nullptr;      // stream every call is ordered on
  cudaStream_t own_stream = nullptr;  // created by qsv_create
  // Growable device scratch (reductions, feeds, tables).
  void* d_scratch = nullptr;
  size_t scratch_bytes = 0;
  // Device status word written by kernels with bounded waits.
  int* d_flag = nullptr;
  // Fault injection for tests (qsv_inject_block_stall): the limit of the stalled wait of
  // the next fused-block launch, 0 when not armed.
  uint64_t inject_stall_ns = 0;
  // Fused-block launches on this state so far: consecutive launches visit the tiles in
  // opposite orders (the next one starts on what the last one wrote, still in L2).
  uint64_t block_launches = 0;
  // Fused-block matrix images: a ring of pinned host staging slots (a slot is reused
  // only after its upload completed, so the host rarely waits for queued kernels) and
  // one device buffer (stream order keeps uploads behind the kernels reading it).
  static constexpr int kImageSlots = 32;
  void* h_img[kImageSlots] = {nullptr};
  size_t h_img_bytes[kImageSlots] = {0};
  cudaEvent_t img_ev[kImageSlots] = {nullptr};
  bool img_busy[kImageSlots] = {false};
  int img_next = 0;
  void* d_images = nullptr;
  size_t d_images_bytes = 0;
  // Pinned staging for host <-> device range copies.
  void* h_stage = nullptr;
  size_t h_stage_bytes = 0;
  char err[512] = {0};
};

namespace qsv {

extern std::atomic<unsigned long long> g_launches;
inline void count_launch(unsigned long long k = 1) {
  g_launches.fetch_add(k, std::memory_order_relaxed);
}

int set_error(qsv_state* s, int code, const char* fmt, ...);
// Out-of-bounds words of each translation unit (bounds-checked build only).
int oob_take_core(unsigned long long* count, unsigned long long* first);
int oob_take_fused(unsigned long long* count, unsigned long long* first);
int oob_take_adjoint(unsigned long long* count, unsigned long long* first);
int oob_take_circuits(unsigned long long* count, unsigned long long* first);
int oob_take_adjtc(unsigned long long* count, unsigned long long* first);
int ensure_scratch(qsv_state* s, size_t bytes);
int check_launch(qsv_state* s, const char* what);
unsigned grid_for(const qsv_state* s, uint64_t work, unsigned per_block = QSV_THREADS,
                  unsigned waves = 16);

// Fused-block geometry for batches of states (qsv_fused.cu), used by the tensor-core
// adjoint: k target qubits in the caller's matrix order (first = most significant);
// tperm_out[t'] is the caller's matrix index of kernel target index t' (64 bytes).
struct FusedGeom;
size_t fused_image_bytes(int k);
int fused_geom_create(int device, int n, int k, const int* qubits, FusedGeom** out, uint8_t* tperm_out);
void fused_geom_destroy(FusedGeom* g);
// True when the geometry's launches want W images with interleaved rows (row nn =
// component nn & 1 of output nn >> 1, the prefix access mode).
bool fused_geom_interleaved(const FusedGeom* g);
// One launch over nsets states of 2^n complex64 amplitudes (psi); state s uses the W
// image at images + s * img_stride.  A bounded wait that gives up sets *flag.
int fused_geom_launch_sets(const FusedGeom* g, float2* psi, int nsets, int n, const void* images,
                           size_t img_stride, int* flag, cudaStream_t stream, int sm_count);
// The adjoint's fused backward pass for one block (k_adj_back): un-computes psi and lambda
// in place with the U^+ images and adds the block's correlation into corr
// ([nsets][128][128] FP64).  Only for geometries where fused_geom_backward_ok holds
// (6 qubits in the direct, prefix or pair access modes); QSV_ERR_UNSUPPORTED otherwise.
bool fused_geom_backward_ok(const FusedGeom* g);
int fused_geom_launch_backward(const FusedGeom* g, float2* psi, float2* lam, double* corr, int nsets, int n,
                               const void* images, size_t img_stride, int* flag, cudaStream_t stream, int sm_count);

// Validates qubit indices (range, duplicates) and converts them to bit positions.
int to_positions(qsv_state* s, int count, const int* qubits, int* pos_out,
                 uint64_t* seen_mask);

template <typename R> struct C2T;
template <> struct C2T<float> { using type = float2; };
template <> struct C2T<double> { using type = double2; };

}  // namespace qsv

#define QSV_CUDA(s, call)                                                          \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess)                                                         \
      return qsv::set_error((s), QSV_ERR_CUDA, "%s: %s", #call,                    \
                            cudaGetErrorString(e_));                               \
  } while (0)

#define QSV_CHECK_HANDLE(s)                                                        \
  do {                                                                             \
    if ((s) == nullptr || (s)->d_amp == nullptr) return QSV_ERR_INVALID;           \
  } while (0)

// ---- device helpers --------------------------------------------------------------

// ---- bounds-checked build ----------------------------------------------------------
// Built with -DQSV_BOUNDS_CHECK (libqsv_checked.so), kernels test every computed state
// index against the state's size before the access.  A bad index is counted in this
// translation unit's device words (the first one kept) and the access is skipped:
// nothing traps.  qsv_bounds_report reads and clears the words of every unit.  In the
// normal build QSV_IN_BOUNDS is the constant true and the tests compile away.
#ifdef QSV_BOUNDS_CHECK
static __device__ unsigned long long qsv_oob_words[2];  // [0] count, [1] first bad index
__device__ __forceinline__ bool qsv_in_bounds(unsigned long long idx, unsigned long long limit) {
  if (idx < limit) return true;
  if (atomicAdd(&qsv_oob_words[0], 1ull) == 0ull) qsv_oob_words[1] = idx;
  return false;
}
#define QSV_IN_BOUNDS(idx, limit) qsv_in_bounds((unsigned long long)(idx), (unsigned long long)(limit))
// This unit's words: adds the count to *count, keeps the first index, clears them.
static inline int qsv_oob_take_unit(unsigned long long* count, unsigned long long* first) {
  unsigned long long w[2] = {0, 0};
  if (cudaMemcpyFromSymbol(w, qsv_oob_words, sizeof(w)) != cudaSuccess) return -1;
  const unsigned long long zero[2] = {0, 0};
  if (cudaMemcpyToSymbol(qsv_oob_words, zero, sizeof(zero)) != cudaSuccess) return -1;
  if (w[0] && !*count) *first = w[1];
  *count += w[0];
  return 0;
}
#else
#define QSV_IN_BOUNDS(idx, limit) true
#endif

// Spreads the bits of g over the positions that are NOT in pos[0..npos) (sorted
// ascending): the inverse of removing those bit positions.
__device__ __forceinline__ uint64_t qsv_insert_zeros(uint64_t g, const int* pos, int npos) {
  for (int i = 0; i < npos; ++i) {
    const int p = pos[i];
    const uint64_t low = g & ((1ull << p) - 1ull);
    g = ((g >> p) << (p + 1)) | low;
  }
  return g;
}

__device__ __forceinline__ float2 qsv_cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 qsv_cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
// acc + a*b
__device__ __forceinline__ float2 qsv_cfma(float2 a, float2 b, float2 acc) {
  acc.x = fmaf(a.x, b.x, acc.x);
  acc.x = fmaf(-a.y, b.y, acc.x);
  acc.y = fmaf(a.x, b.y, acc.y);
  acc.y = fmaf(a.y, b.x, acc.y);
  return acc;
}
__device__ __forceinline__ double2 qsv_cfma(double2 a, double2 b, double2 acc) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
  return acc;
}
