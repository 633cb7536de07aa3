// Batched state vectors and the adjoint-method gradient.
//
// A batch is `nsets` independent states of 2^n amplitudes stored back to back in one
// device buffer owned by the caller (e.g. a torch tensor of shape [nsets, 2^n]).  One
// launch applies a single-qubit gate to every state of the batch, each with its own 2x2
// matrix (the gate's angle differs per parameter set).
//
// Adjoint method for E(theta) = <psi| O |psi>, psi = U_G ... U_1 |psi_0>, with
// O = sum_i Z_i:
//   lambda = O psi_G;  for g = G .. 1:  [if U_g = exp(-i theta P / 2):
//   dE/dtheta_g = Im <lambda| P |psi_g>];  psi <- U_g^+ psi;  lambda <- U_g^+ lambda.
// qsv_batch_adjoint_step does one g for every state of the batch in one pass over psi
// and lambda: the generator product is reduced per state before both vectors are
// un-computed.  Three vectors per parameter set are never needed: psi and lambda only.
//
// Reductions of complex64 batches accumulate per thread in double-float (FP32 pairs)
// and across threads / blocks in FP64, like the measurement reductions.

#include <algorithm>

#include "qsv_internal.cuh"

using namespace qsv;

namespace {

template <typename R>
using CT = typename C2T<R>::type;

struct DF2 {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float a) {
    const float t = hi + a;
    const float z = t - hi;
    lo += (hi - (t - z)) + (a - z);
    hi = t;
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

template <typename R>
struct RedAcc;
template <>
struct RedAcc<float> {
  DF2 d;
  __device__ __forceinline__ void add(float v) { d.add(v); }
  __device__ __forceinline__ double value() const { return d.value(); }
};
template <>
struct RedAcc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double v) { s += v; }
  __device__ __forceinline__ double value() const { return s; }
};

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double block_sum_d(double v, double* sh) {
  v = warp_sum_d(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
    r = warp_sum_d(r);
  }
  return r;
}

template <typename R>
__device__ __forceinline__ CT<R> cconj(CT<R> a) {
  a.y = -a.y;
  return a;
}

struct BatchGate {
  uint64_t ngroups;  // 2^(n - 1 - ncontrols) pairs per state
  uint64_t ctrl;     // control mask (OR-ed into every pair base)
  int p;             // target bit position
  int npos;
  int pos[2];        // target (+ control) positions, ascending
  int n;
  int nsets;
};

// psi[s] <- M_s psi[s] on the target (pairs with the control bit set).
template <typename R>
__global__ void __launch_bounds__(QSV_THREADS)
    k_batch_1q(CT<R>* __restrict__ psi, const CT<R>* __restrict__ mats, const BatchGate a) {
  const int s = blockIdx.y;
  CT<R>* v = psi + ((uint64_t)s << a.n);
  const CT<R> m00 = mats[4 * s], m01 = mats[4 * s + 1], m10 = mats[4 * s + 2], m11 = mats[4 * s + 3];
  const uint64_t hi = 1ull << a.p;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < a.ngroups; g += stride) {
    const uint64_t i0 = qsv_insert_zeros(g, a.pos, a.npos) | a.ctrl;
    const CT<R> x = v[i0], y = v[i0 + hi];
    CT<R> o0, o1;
    o0.x = R(0); o0.y = R(0); o1 = o0;
    o0 = qsv_cfma(m00, x, o0);
    o0 = qsv_cfma(m01, y, o0);
    o1 = qsv_cfma(m10, x, o1);
    o1 = qsv_cfma(m11, y, o1);
    v[i0] = o0;
    v[i0 + hi] = o1;
  }
}

// lambda = (sum_i Z_i) psi; partial[s][block] = sum (n - 2 popcount(x)) |psi_x|^2.
template <typename R>
__global__ void __launch_bounds__(QSV_THREADS)
    k_batch_sumz(const CT<R>* __restrict__ psi, CT<R>* __restrict__ lam, int n, double* __restrict__ partial) {
  __shared__ double sh[32];
  const int s = blockIdx.y;
  const uint64_t off = (uint64_t)s << n;
  const uint64_t total = 1ull << n;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  RedAcc<R> acc;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += stride) {
    const CT<R> v = psi[off + i];
    const R w = R(n - 2 * __popcll(i));
    CT<R> l;
    l.x = w * v.x;
    l.y = w * v.y;
    lam[off + i] = l;
    acc.add(w * (v.x * v.x + v.y * v.y));
  }
  const double r = block_sum_d(acc.value(), sh);
  if (threadIdx.x == 0) partial[(uint64_t)s * gridDim.x + blockIdx.x] = r;
}

// One backward step: optional generator reduction Im<lambda|P|psi> (P = Y or Z on the
// target; uncontrolled gates only), then psi <- M_s psi, lambda <- M_s lambda with
// M_s = U_s^+ supplied by the caller.
template <typename R>
__global__ void __launch_bounds__(QSV_THREADS)
    k_batch_adjoint(CT<R>* __restrict__ psi, CT<R>* __restrict__ lam, const CT<R>* __restrict__ mats,
                    const BatchGate a, int gen, double* __restrict__ partial) {
  __shared__ double sh[32];
  const int s = blockIdx.y;
  const uint64_t off = (uint64_t)s << a.n;
  CT<R>* pv = psi + off;
  CT<R>* lv = lam + off;
  const CT<R> m00 = mats[4 * s], m01 = mats[4 * s + 1], m10 = mats[4 * s + 2], m11 = mats[4 * s + 3];
  const uint64_t hi = 1ull << a.p;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  RedAcc<R> acc;
  for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < a.ngroups; g += stride) {
    const uint64_t i0 = qsv_insert_zeros(g, a.pos, a.npos) | a.ctrl;
    const CT<R> x = pv[i0], y = pv[i0 + hi];
    const CT<R> l0 = lv[i0], l1 = lv[i0 + hi];
    if (gen == 2) {
      // Im[conj(l0) x - conj(l1) y]
      acc.add((l0.x * x.y - l0.y * x.x) - (l1.x * y.y - l1.y * y.x));
    } else if (gen == 1) {
      // Y x = (-i y, i x): Im[conj(l0)(-i y) + conj(l1)(i x)] = -Re[conj(l0) y] + Re[conj(l1) x]
      acc.add((l1.x * x.x + l1.y * x.y) - (l0.x * y.x + l0.y * y.y));
    }
    CT<R> o0, o1, q0, q1;
    o0.x = R(0); o0.y = R(0); o1 = o0; q0 = o0; q1 = o0;
    o0 = qsv_cfma(m00, x, o0);
    o0 = qsv_cfma(m01, y, o0);
    o1 = qsv_cfma(m10, x, o1);
    o1 = qsv_cfma(m11, y, o1);
    q0 = qsv_cfma(m00, l0, q0);
    q0 = qsv_cfma(m01, l1, q0);
    q1 = qsv_cfma(m10, l0, q1);
    q1 = qsv_cfma(m11, l1, q1);
    pv[i0] = o0;
    pv[i0 + hi] = o1;
    lv[i0] = q0;
    lv[i0 + hi] = q1;
  }
  if (gen) {
    const double r = block_sum_d(acc.value(), sh);
    if (threadIdx.x == 0) partial[(uint64_t)s * gridDim.x + blockIdx.x] = r;
  }
}

// out[s * out_stride] = sum_b partial[s * nblk + b] (FP64, Neumaier).
__global__ void k_batch_finish(const double* __restrict__ partial, int nblk, int nsets, double* __restrict__ out,
                               int out_stride) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsets) return;
  double sum = 0.0, c = 0.0;
  for (int b = 0; b < nblk; ++b) {
    const double x = partial[(uint64_t)s * nblk + b];
    const double t = sum + x;
    c += (fabs(sum) >= fabs(x)) ? (sum - t) + x : (x - t) + sum;
    sum = t;
  }
  out[(uint64_t)s * out_stride] = sum + c;
}

template <typename R>
__global__ void k_batch_zero(CT<R>* psi, int n, int nsets) {
  const uint64_t total = (uint64_t)nsets << n;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += stride) {
    CT<R> v;
    v.x = ((i & ((1ull << n) - 1ull)) == 0) ? R(1) : R(0);
    v.y = R(0);
    psi[i] = v;
  }
}

int g_sms = 0;
int sms() {
  if (!g_sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_sms < 1) g_sms = 1;
  }
  return g_sms;
}

int gate_args(int n, int nsets, int target, int control, BatchGate& a) {
  if (n < 2 || n > QSV_MAXN || nsets < 1 || nsets > 65535)
    return set_error(nullptr, QSV_ERR_INVALID, "bad batch shape n=%d nsets=%d", n, nsets);
  if (target < 0 || target >= n || control >= n || control == target)
    return set_error(nullptr, QSV_ERR_INVALID, "bad target %d / control %d for n=%d", target, control, n);
  a.n = n;
  a.nsets = nsets;
  a.p = n - 1 - target;
  a.npos = 1;
  a.pos[0] = a.p;
  a.ctrl = 0;
  if (control >= 0) {
    const int cp = n - 1 - control;
    a.ctrl = 1ull << cp;
    a.pos[1] = cp;
    a.npos = 2;
    if (a.pos[0] > a.pos[1]) std::swap(a.pos[0], a.pos[1]);
  }
  a.ngroups = 1ull << (n - a.npos);
  return QSV_OK;
}

// Blocks per state: enough to fill the GPU across the whole batch.
unsigned blocks_per_set(uint64_t work, int nsets) {
  uint64_t want = (uint64_t)sms() * 16 / (uint64_t)nsets;
  if (want < 1) want = 1;
  const uint64_t need = (work + QSV_THREADS - 1) / QSV_THREADS;
  return (unsigned)std::max<uint64_t>(1, std::min(want, need));
}

int launch_check(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(nullptr, QSV_ERR_CUDA, "%s launch: %s", what, cudaGetErrorString(e));
  count_launch();
  return QSV_OK;
}

}  // namespace

extern "C" {

int qsv_batch_reset(void* psi, int nsets, int n, int dtype, void* stream) {
  if (!psi || n < 1 || n > QSV_MAXN || nsets < 1) return set_error(nullptr, QSV_ERR_INVALID, "bad batch");
  const unsigned grid = (unsigned)std::min<uint64_t>((((uint64_t)nsets << n) + QSV_THREADS - 1) / QSV_THREADS,
                                                     (uint64_t)sms() * 16);
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == QSV_C64)
    k_batch_zero<float><<<grid, QSV_THREADS, 0, st>>>((float2*)psi, n, nsets);
  else if (dtype == QSV_C128)
    k_batch_zero<double><<<grid, QSV_THREADS, 0, st>>>((double2*)psi, n, nsets);
  else
    return set_error(nullptr, QSV_ERR_INVALID, "unknown dtype %d", dtype);
  return launch_check("batch_reset");
}

int qsv_batch_apply_1q(void* psi, int nsets, int n, int dtype, int target, int control, const void* mats,
                       void* stream) {
  if (!psi || !mats) return set_error(nullptr, QSV_ERR_INVALID, "null pointer");
  BatchGate a;
  int rc = gate_args(n, nsets, target, control, a);
  if (rc) return rc;
  dim3 grid(blocks_per_set(a.ngroups, nsets), (unsigned)nsets);
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == QSV_C64)
    k_batch_1q<float><<<grid, QSV_THREADS, 0, st>>>((float2*)psi, (const float2*)mats, a);
  else if (dtype == QSV_C128)
    k_batch_1q<double><<<grid, QSV_THREADS, 0, st>>>((double2*)psi, (const double2*)mats, a);
  else
    return set_error(nullptr, QSV_ERR_INVALID, "unknown dtype %d", dtype);
  return launch_check("batch_apply_1q");
}

int qsv_batch_observable_sumz(const void* psi, void* lam, int nsets, int n, int dtype, double* energies,
                              double* scratch, size_t scratch_doubles, void* stream) {
  if (!psi || !lam || !energies || !scratch) return set_error(nullptr, QSV_ERR_INVALID, "null pointer");
  if (n < 1 || n > QSV_MAXN || nsets < 1 || nsets > 65535) return set_error(nullptr, QSV_ERR_INVALID, "bad batch");
  const unsigned nb = blocks_per_set(1ull << n, nsets);
  if ((size_t)nb * nsets > scratch_doubles)
    return set_error(nullptr, QSV_ERR_INVALID, "scratch of %zu doubles < %zu needed", scratch_doubles,
                     (size_t)nb * nsets);
  dim3 grid(nb, (unsigned)nsets);
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == QSV_C64)
    k_batch_sumz<float><<<grid, QSV_THREADS, 0, st>>>((const float2*)psi, (float2*)lam, n, scratch);
  else if (dtype == QSV_C128)
    k_batch_sumz<double><<<grid, QSV_THREADS, 0, st>>>((const double2*)psi, (double2*)lam, n, scratch);
  else
    return set_error(nullptr, QSV_ERR_INVALID, "unknown dtype %d", dtype);
  int rc = launch_check("batch_sumz");
  if (rc) return rc;
  k_batch_finish<<<(nsets + 127) / 128, 128, 0, st>>>(scratch, (int)nb, nsets, energies, 1);
  return launch_check("batch_finish");
}

int qsv_batch_adjoint_step(void* psi, void* lam, int nsets, int n, int dtype, int target, int control,
                           const void* mats_dagger, int generator, double* grads, int grad_stride, double* scratch,
                           size_t scratch_doubles, void* stream) {
  if (!psi || !lam || !mats_dagger) return set_error(nullptr, QSV_ERR_INVALID, "null pointer");
  if (generator < 0 || generator > 2) return set_error(nullptr, QSV_ERR_INVALID, "generator %d", generator);
  if (generator && (control >= 0 || !grads || !scratch))
    return set_error(nullptr, QSV_ERR_INVALID, "generator needs an uncontrolled gate, grads and scratch");
  BatchGate a;
  int rc = gate_args(n, nsets, target, control, a);
  if (rc) return rc;
  const unsigned nb = blocks_per_set(a.ngroups, nsets);
  if (generator && (size_t)nb * nsets > scratch_doubles)
    return set_error(nullptr, QSV_ERR_INVALID, "scratch of %zu doubles < %zu needed", scratch_doubles,
                     (size_t)nb * nsets);
  dim3 grid(nb, (unsigned)nsets);
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == QSV_C64)
    k_batch_adjoint<float><<<grid, QSV_THREADS, 0, st>>>((float2*)psi, (float2*)lam, (const float2*)mats_dagger, a,
                                                         generator, scratch);
  else if (dtype == QSV_C128)
    k_batch_adjoint<double><<<grid, QSV_THREADS, 0, st>>>((double2*)psi, (double2*)lam,
                                                          (const double2*)mats_dagger, a, generator, scratch);
  else
    return set_error(nullptr, QSV_ERR_INVALID, "unknown dtype %d", dtype);
  rc = launch_check("batch_adjoint");
  if (rc || !generator) return rc;
  k_batch_finish<<<(nsets + 127) / 128, 128, 0, st>>>(scratch, (int)nb, nsets, grads, grad_stride);
  return launch_check("batch_finish");
}

}  // extern "C"
