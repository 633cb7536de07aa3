// libqsv core: handle lifetime, state preparation and readout, the per-gate HBM
// kernels (dense / diagonal / monomial / register swap), measurement reductions and
// the function-oracle permutation.  The tensor-core fused-block path lives in
// qsv_fused.cu.
//
// Layout: one dense vector of 2^n amplitudes (float2 or double2) in HBM; amplitude
// index bit (n-1-q) is qubit q (qubit 0 = most significant bit), the reference's
// convention (qip/ext/kronprod.pyx:168, 187-189).  Updates are in place.

#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <mutex>
#include <thread>
#include <new>
#include <type_traits>
#include <vector>

#include "qsv_internal.cuh"

namespace qsv {

std::atomic<unsigned long long> g_launches{0};
static char g_global_err[512] = {0};
static std::mutex g_global_err_mu;

int set_error(qsv_state* s, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (s) {
    memcpy(s->err, buf, sizeof(buf));
  } else {
    std::lock_guard<std::mutex> lk(g_global_err_mu);
    memcpy(g_global_err, buf, sizeof(buf));
  }
  return code;
}

int ensure_scratch(qsv_state* s, size_t bytes) {
  if (bytes <= s->scratch_bytes) return QSV_OK;
  size_t want = std::max(bytes, s->scratch_bytes * 2);
  want = (want + 255) & ~size_t(255);
  if (s->d_scratch) {
    // The old scratch may still be read by queued kernels.
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return set_error(s, QSV_ERR_CUDA, "sync: %s", cudaGetErrorString(e));
    cudaFree(s->d_scratch);
    s->d_scratch = nullptr;
    s->scratch_bytes = 0;
  }
  if (cudaMalloc(&s->d_scratch, want) != cudaSuccess) {
    cudaGetLastError();
    return set_error(s, QSV_ERR_OOM, "scratch allocation of %zu bytes failed", want);
  }
  s->scratch_bytes = want;
  return QSV_OK;
}

int check_launch(qsv_state* s, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(s, QSV_ERR_CUDA, "%s launch: %s", what, cudaGetErrorString(e));
  count_launch();
  return QSV_OK;
}

unsigned grid_for(const qsv_state* s, uint64_t work, unsigned per_block, unsigned waves) {
  uint64_t blocks = (work + per_block - 1) / per_block;
  uint64_t cap = (uint64_t)std::max(1, s->sm_count) * waves;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  return (unsigned)blocks;
}

int to_positions(qsv_state* s, int count, const int* qubits, int* pos_out, uint64_t* seen_mask) {
  if (count < 0 || count > QSV_MAXQ) return set_error(s, QSV_ERR_INVALID, "too many qubits (%d)", count);
  if (count > 0 && qubits == nullptr) return set_error(s, QSV_ERR_INVALID, "null qubit list");
  for (int i = 0; i < count; ++i) {
    const int q = qubits[i];
    if (q < 0 || q >= s->n)
      return set_error(s, QSV_ERR_INVALID, "qubit index %d out of range for n=%d", q, s->n);
    const int p = s->n - 1 - q;
    if (*seen_mask & (1ull << p)) return set_error(s, QSV_ERR_INVALID, "qubit %d repeated", q);
    *seen_mask |= 1ull << p;
    pos_out[i] = p;
  }
  return QSV_OK;
}

}  // namespace qsv

using namespace qsv;

// ======================================================================================
// Kernels
// ======================================================================================
namespace {

template <typename R>
using CT = typename C2T<R>::type;

template <typename R>
__global__ void k_set_basis(CT<R>* psi, uint64_t index) {
  CT<R> one;
  one.x = R(1);
  one.y = R(0);
  psi[index] = one;
}

// ---- product state: amp[i] = prod_g feed_g[sub_g(i)] (qip/backend.py:94-101) ---------
struct ProductArgs {
  uint64_t total;
  uint64_t unfed_mask;
  int ngroups;
  int nq;                       // total fed qubits
  int size[QSV_MAXQ];           // qubits per group
  int pos[QSV_MAXQ];            // bit positions, group by group, first = MSB of the group
  uint64_t feed_off[QSV_MAXQ];  // offset of group g's vector in the feed buffer
};

template <typename R>
__global__ void __launch_bounds__(QSV_THREADS)
    k_product(CT<R>* __restrict__ psi, const double2* __restrict__ feeds,
              const __grid_constant__ ProductArgs a) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < a.total; i += stride) {
    CT<R> out;
    if (i & a.unfed_mask) {
      out.x = R(0);
      out.y = R(0);
    } else {
      double2 acc = make_double2(1.0, 0.0);
      int q = 0;
      for (int g = 0; g < a.ngroups; ++g) {
        uint64_t sub = 0;
        for (int j = 0; j < a.size[g]; ++j, ++q) sub = (sub << 1) | ((i >> a.pos[q]) & 1ull);
        const double2 f = feeds[a.feed_off[g] + sub];
        acc = make_double2(acc.x * f.x - acc.y * f.y, acc.x * f.y + acc.y * f.x);
      }
      out.x = R(acc.x);
      out.y = R(acc.y);
    }
    psi[i] = out;
  }
}

template <typename R>
__global__ void __launch_bounds__(QSV_THREADS)
    k_add_range(CT<R>* __restrict__ psi, const CT<R>* __restrict__ src, uint64_t count) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < count; i += stride) {
    CT<R> a = psi[i];
    const CT<R> b = src[i];
    a.x += b.x;
    a.y += b.y;
    psi[i] = a;
  }
}

// ---- dense k-qubit gate with controls -------------------------------------------------
template <typename R, int K>
struct DenseArgs {
  uint64_t ngroups;
  uint64_t ctrl;               // OR-ed into every group base (controls == 1)
  uint64_t off[1 << K];        // state offset of matrix index j (targets[0] = MSB)
  int npos;
  int pos[QSV_MAXQ];           // target+control bit positions, ascending
  CT<R> m[(1 << K) * (1 << K)];  // row-major
};

// Vector loads/stores of 2^VB adjacent amplitudes (complex64; VB = 1: 16 bytes, VB = 2:
// 32 bytes).  Used when matrix index bits 0..VB-1 are address bits 0..VB-1 (the host
// orders the targets so), which turns a warp's 8-byte accesses spread over 2^VB times
// as many cache lines into dense ones.
template <int VB>
__device__ __forceinline__ void ld_amps(const float2* p, float2* v) {
  if constexpr (VB == 2) {
    float f[8];
    asm volatile("ld.global.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=f"(f[0]), "=f"(f[1]), "=f"(f[2]), "=f"(f[3]), "=f"(f[4]), "=f"(f[5]), "=f"(f[6]), "=f"(f[7])
                 : "l"(p));
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] = make_float2(f[2 * i], f[2 * i + 1]);
  } else {
    const float4 x = *reinterpret_cast<const float4*>(p);
    v[0] = make_float2(x.x, x.y);
    v[1] = make_float2(x.z, x.w);
  }
}
template <int VB>
__device__ __forceinline__ void st_amps(float2* p, const float2* v) {
  if constexpr (VB == 2) {
    asm volatile("st.global.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(p), "f"(v[0].x), "f"(v[0].y),
                 "f"(v[1].x), "f"(v[1].y), "f"(v[2].x), "f"(v[2].y), "f"(v[3].x), "f"(v[3].y)
                 : "memory");
  } else {
    *reinterpret_cast<float4*>(p) = make_float4(v[0].x, v[0].y, v[1].x, v[1].y);
  }
}

template <typename R, int K, int VB>
__global__ void __launch_bounds__(QSV_THREADS)
    k_dense(CT<R>* __restrict__ psi, const __grid_constant__ DenseArgs<R, K> a) {
  constexpr int D = 1 << K;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t lim = a.ngroups << a.npos;  // the state's size
  for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < a.ngroups; g += stride) {
    const uint64_t base = qsv_insert_zeros(g, a.pos, a.npos) | a.ctrl;
    bool ok = true;
#pragma unroll
    for (int j = 0; j < D; j += 1 << VB) ok = ok && QSV_IN_BOUNDS(base + a.off[j] + (1u << VB) - 1u, lim);
    if (!ok) continue;
    CT<R> v[D];
    if constexpr (VB > 0) {
      static_assert(K <= 3 && VB <= K, "vector path covers up to 3 targets");
#pragma unroll
      for (int j = 0; j < D; j += 1 << VB) ld_amps<VB>(psi + base + a.off[j], &v[j]);
      CT<R> o[D];
#pragma unroll
      for (int r = 0; r < D; ++r) {
        o[r].x = R(0);
        o[r].y = R(0);
#pragma unroll
        for (int c = 0; c < D; ++c) o[r] = qsv_cfma(a.m[r * D + c], v[c], o[r]);
      }
#pragma unroll
      for (int j = 0; j < D; j += 1 << VB) st_amps<VB>(psi + base + a.off[j], &o[j]);
      continue;
    } else {
#pragma unroll
      for (int j = 0; j < D; ++j) v[j] = psi[base + a.off[j]];
    }
    if constexpr (K <= 3) {
#pragma unroll
      for (int r = 0; r < D; ++r) {
        CT<R> acc;
        acc.x = R(0);
        acc.y = R(0);
#pragma unroll
        for (int c = 0; c < D; ++c) acc = qsv_cfma(a.m[r * D + c], v[c], acc);
        psi[base + a.off[r]] = acc;
      }
    } else {
#pragma unroll 1
      for (int r = 0; r < D; ++r) {
        CT<R> acc;
        acc.x = R(0);
        acc.y = R(0);
#pragma unroll
        for (int c = 0; c < D; ++c) acc = qsv_cfma(a.m[r * D + c], v[c], acc);
        psi[base + a.off[r]] = acc;
      }
    }
  }
}

// Specialised single-qubit dense gate without controls: the most common plain pass.
template <typename R>
struct Dense1Args {
  uint64_t ngroups;
  int p;  // target bit position
  CT<R> m00, m01, m10, m11;
};

// REAL: the matrix has no imaginary parts (H, RY, ...): half the multiplies, which
// matters for complex128 where the FP64 pipe, not HBM, bounds the pass on GB300.
template <typename R, bool REAL>
__global__ void __launch_bounds__(QSV_THREADS)
    k_dense1(CT<R>* __restrict__ psi, const __grid_constant__ Dense1Args<R> a) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t lowmask = (1ull << a.p) - 1ull;
  const uint64_t hi = 1ull << a.p;
  for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < a.ngroups; g += stride) {
    const uint64_t i0 = ((g >> a.p) << (a.p + 1)) | (g & lowmask);
    if (!QSV_IN_BOUNDS(i0 + hi, a.ngroups << 1)) continue;
    const CT<R> x = psi[i0];
    const CT<R> y = psi[i0 + hi];
    CT<R> o0, o1;
    if constexpr (REAL) {
      o0.x = a.m00.x * x.x + a.m01.x * y.x;
      o0.y = a.m00.x * x.y + a.m01.x * y.y;
      o1.x = a.m10.x * x.x + a.m11.x * y.x;
      o1.y = a.m10.x * x.y + a.m11.x * y.y;
    } else {
      o0.x = R(0); o0.y = R(0); o1 = o0;
      o0 = qsv_cfma(a.m00, x, o0);
      o0 = qsv_cfma(a.m01, y, o0);
      o1 = qsv_cfma(a.m10, x, o1);
      o1 = qsv_cfma(a.m11, y, o1);
    }
    psi[i0] = o0;
    psi[i0 + hi] = o1;
  }
}

// ---- diagonal: only entries != 1 are touched ------------------------------------------
constexpr int QSV_MAXDIAG = 256;
template <typename R>
struct DiagArgs {
  uint64_t ngroups;
  uint64_t ctrl;
  int npos;
  int pos[QSV_MAXQ];
  int nent;
  uint64_t off[QSV_MAXDIAG];
  CT<R> ph[QSV_MAXDIAG];
};

template <typename R>
__global__ void __launch_bounds__(QSV_THREADS)
    k_diag(CT<R>* __restrict__ psi, const __grid_constant__ DiagArgs<R> a) {
  // Four groups per thread (stride apart, so a warp's accesses stay adjacent), their
  // loads issued together: one amplitude per thread in flight is too little to keep
  // HBM busy when a gate touches a single entry.
  constexpr int U = 4;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t g0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g0 < a.ngroups; g0 += U * stride) {
    uint64_t base[U];
#pragma unroll
    for (int u = 0; u < U; ++u) base[u] = qsv_insert_zeros(g0 + u * stride, a.pos, a.npos) | a.ctrl;
    for (int e = 0; e < a.nent; ++e) {
      CT<R> x[U];
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (g0 + u * stride < a.ngroups && QSV_IN_BOUNDS(base[u] + a.off[e], a.ngroups << a.npos))
          x[u] = psi[base[u] + a.off[e]];
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (g0 + u * stride < a.ngroups && QSV_IN_BOUNDS(base[u] + a.off[e], a.ngroups << a.npos))
          psi[base[u] + a.off[e]] = qsv_cmul(a.ph[e], x[u]);
    }
  }
}

// ---- monomial: out[r] = phase[r] * in[perm[r]] ----------------------------------------
template <typename R, int K>
struct MonoArgs {
  uint64_t ngroups;
  uint64_t ctrl;
  int npos;
  int pos[QSV_MAXQ];
  uint64_t off[1 << K];
  int perm[1 << K];
  unsigned exact;  // bit r set: phase[r] == 1, move without arithmetic
  CT<R> ph[1 << K];
};

// PURE: every phase is exactly 1, so the gate only moves amplitudes (no arithmetic is
// compiled in at all, bit-exact and bandwidth-bound in either precision).
template <typename R, int K, bool PURE>
__global__ void __launch_bounds__(QSV_THREADS)
    k_mono(CT<R>* __restrict__ psi, const __grid_constant__ MonoArgs<R, K> a) {
  constexpr int D = 1 << K;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < a.ngroups; g += stride) {
    const uint64_t base = qsv_insert_zeros(g, a.pos, a.npos) | a.ctrl;
    bool ok = true;
#pragma unroll
    for (int j = 0; j < D; ++j) ok = ok && QSV_IN_BOUNDS(base + a.off[j], a.ngroups << a.npos);
    if (!ok) continue;
    CT<R> v[D];
#pragma unroll
    for (int j = 0; j < D; ++j) v[j] = psi[base + a.off[j]];
#pragma unroll
    for (int r = 0; r < D; ++r) {
      CT<R> x = v[0];
#pragma unroll
      for (int c = 1; c < D; ++c)
        if (a.perm[r] == c) x = v[c];
      if constexpr (!PURE) {
        if (!((a.exact >> r) & 1u)) x = qsv_cmul(a.ph[r], x);
      }
      psi[base + a.off[r]] = x;
    }
  }
}

// ---- register swap (SwapMat) -----------------------------------------------------------
struct SwapArgs {
  uint64_t nitems;  // 2^(n - ncontrols)
  uint64_t ctrl;
  int ncp;
  int cpos[QSV_MAXQ];  // control positions ascending
  int m;
  int apos[QSV_MAXQ / 2];  // register a, first = MSB
  int bpos[QSV_MAXQ / 2];
};

// Single-qubit swap (m = 1): one item per exchanged pair (a = 1, b = 0) <-> (a = 0,
// b = 1), two items per thread.  pos holds a, b and the controls, ascending.
struct Swap1Args {
  uint64_t nitems;  // 2^(n - 2 - ncontrols)
  uint64_t ctrl;    // controls | bit a
  uint64_t flip;    // bit a | bit b
  int npos;
  int pos[QSV_MAXQ];
};

template <typename R>
__global__ void __launch_bounds__(QSV_THREADS)
    k_swap1(CT<R>* __restrict__ psi, const __grid_constant__ Swap1Args a) {
  constexpr int U = 2;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t t0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t0 < a.nitems; t0 += U * stride) {
    uint64_t idx[U];
    CT<R> x[U], y[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      idx[u] = qsv_insert_zeros(t0 + u * stride, a.pos, a.npos) | a.ctrl;
      if (t0 + u * stride < a.nitems && QSV_IN_BOUNDS(idx[u] | a.flip, a.nitems << a.npos)) {
        x[u] = psi[idx[u]];
        y[u] = psi[idx[u] ^ a.flip];
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (t0 + u * stride < a.nitems && QSV_IN_BOUNDS(idx[u] | a.flip, a.nitems << a.npos)) {
        psi[idx[u]] = y[u];
        psi[idx[u] ^ a.flip] = x[u];
      }
  }
}

template <typename R>
__global__ void __launch_bounds__(QSV_THREADS)
    k_swap(CT<R>* __restrict__ psi, const __grid_constant__ SwapArgs a) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < a.nitems; t += stride) {
    const uint64_t idx = qsv_insert_zeros(t, a.cpos, a.ncp) | a.ctrl;
    unsigned x = 0, y = 0;
    uint64_t flip = 0;
    for (int j = 0; j < a.m; ++j) {
      const unsigned xb = (idx >> a.apos[j]) & 1u;
      const unsigned yb = (idx >> a.bpos[j]) & 1u;
      x = (x << 1) | xb;
      y = (y << 1) | yb;
      if (xb != yb) flip |= (1ull << a.apos[j]) | (1ull << a.bpos[j]);
    }
    if (x < y) {
      const uint64_t partner = idx ^ flip;
      if (!QSV_IN_BOUNDS(idx | flip, a.nitems << a.ncp)) continue;
      const CT<R> u = psi[idx];
      const CT<R> w = psi[partner];
      psi[idx] = w;
      psi[partner] = u;
    }
  }
}

// ---- measurement reductions ---------------------------------------------------------------
// Precision plan.  GB300 has little FP64 throughput, so per-element work stays off the
// FP64 pipe where the state allows it: for complex64 states each |a|^2 is formed as an
// exact FP32 pair (products by fma, then TwoSum of the two squares) and accumulated per
// thread in double-float (Knuth TwoSum, ~48-bit precision at FP32 rate).  complex128
// states accumulate in FP64.  Thread partials are combined in FP64 through a pairwise
// tree and block partials with Neumaier compensation, so the result carries FP64-level
// error whatever the state size.

// Neumaier-compensated FP64 accumulation.
struct Acc {
  double s = 0.0, c = 0.0;
  __device__ __forceinline__ void add(double x) {
    const double t = s + x;
    if (fabs(s) >= fabs(x))
      c += (s - t) + x;
    else
      c += (x - t) + s;
    s = t;
  }
  __device__ __forceinline__ double value() const { return s + c; }
};

// Double-float accumulator: value = hi + lo.
struct DF {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float a) {
    const float t = hi + a;
    const float z = t - hi;
    lo += (hi - (t - z)) + (a - z);
    hi = t;
  }
  __device__ __forceinline__ void merge(const DF& o) {
    add(o.hi);
    lo += o.lo;
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

template <typename R>
struct Sq;

template <>
struct Sq<float> {
  struct Term {
    float s, e;  // |v|^2 = s + e (to ~2^-46 relative)
  };
  static __device__ __forceinline__ Term term(float2 v) {
    const float px = v.x * v.x, py = v.y * v.y;
    const float ex = fmaf(v.x, v.x, -px), ey = fmaf(v.y, v.y, -py);
    const float t = px + py;
    const float z = t - px;
    const float e2 = (px - (t - z)) + (py - z);
    return {t, ex + ey + e2};
  }
  struct Accum {
    DF d;
    __device__ __forceinline__ void add(const Term& t) {
      d.add(t.s);
      d.lo += t.e;
    }
    __device__ __forceinline__ void merge(const Accum& o) { d.merge(o.d); }
    __device__ __forceinline__ double value() const { return d.value(); }
  };
};

template <>
struct Sq<double> {
  using Term = double;
  static __device__ __forceinline__ Term term(double2 v) { return fma(v.x, v.x, v.y * v.y); }
  struct Accum {
    double s = 0.0;
    __device__ __forceinline__ void add(Term t) { s += t; }
    __device__ __forceinline__ void merge(const Accum& o) { s += o.s; }
    __device__ __forceinline__ double value() const { return s; }
  };
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of one double per thread (result valid in thread 0).
__device__ __forceinline__ double block_sum(double v, double* sh) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
    r = warp_sum(r);
  }
  return r;
}

struct ProbArgs {
  uint64_t nrest;   // 2^(n-m) amplitudes per outcome
  uint64_t chunk;   // amplitudes per block along the rest index
  uint64_t nchunks;
  uint64_t nbins;
  int m;
  int npos;
  int pos[QSV_MAXQ];          // measured positions ascending (zero insertion)
  uint64_t binbit[QSV_MAXQ];  // outcome bit j -> state mask of qubits[j]
};

// partial[bin * nchunks + chunk] = sum over one chunk of the rest index.
template <typename R>
__global__ void __launch_bounds__(QSV_THREADS)
    k_probs_partial(const CT<R>* __restrict__ psi, const __grid_constant__ ProbArgs a,
                    double* __restrict__ partial) {
  using S = Sq<R>;
  __shared__ double sh[32];
  const uint64_t blk = blockIdx.x + (uint64_t)blockIdx.y * gridDim.x;
  if (blk >= a.nbins * a.nchunks) return;
  const uint64_t bin = blk / a.nchunks;
  const uint64_t chunk = blk - bin * a.nchunks;
  uint64_t binbase = 0;
  for (int j = 0; j < a.m; ++j)
    if ((bin >> j) & 1ull) binbase |= a.binbit[j];
  const uint64_t r0 = chunk * a.chunk;
  const uint64_t r1 = min(r0 + a.chunk, a.nrest);
  const uint64_t bd = blockDim.x;
  typename S::Accum acc[4];
  uint64_t r = r0 + threadIdx.x;
  for (; r + 3 * bd < r1; r += 4 * bd) {
    CT<R> v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint64_t i = qsv_insert_zeros(r + u * bd, a.pos, a.npos) | binbase;
      v[u] = QSV_IN_BOUNDS(i, a.nrest << a.npos) ? psi[i] : CT<R>{};
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) acc[u].add(S::term(v[u]));
  }
  for (; r < r1; r += bd) {
    const uint64_t i = qsv_insert_zeros(r, a.pos, a.npos) | binbase;
    if (QSV_IN_BOUNDS(i, a.nrest << a.npos)) acc[0].add(S::term(psi[i]));
  }
  acc[0].merge(acc[1]);
  acc[2].merge(acc[3]);
  acc[0].merge(acc[2]);
  const double tot = block_sum(acc[0].value(), sh);
  if (threadIdx.x == 0) partial[blk] = tot;
}

// One thread per outcome, looping over the rest index (used when outcomes are many).
template <typename R>
__global__ void __launch_bounds__(QSV_THREADS)
    k_probs_perbin(const CT<R>* __restrict__ psi, const __grid_constant__ ProbArgs a,
                   double* __restrict__ out) {
  using S = Sq<R>;
  const uint64_t bin = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (bin >= a.nbins) return;
  uint64_t binbase = 0;
  for (int j = 0; j < a.m; ++j)
    if ((bin >> j) & 1ull) binbase |= a.binbit[j];
  typename S::Accum acc;
  for (uint64_t r = 0; r < a.nrest; ++r) {
    const uint64_t i = qsv_insert_zeros(r, a.pos, a.npos) | binbase;
    if (QSV_IN_BOUNDS(i, a.nrest << a.npos)) acc.add(S::term(psi[i]));
  }
  out[bin] = acc.value();
}

// out[b] = compensated sum of partial[b*nchunks .. +nchunks), one warp per outcome.
__global__ void __launch_bounds__(QSV_THREADS)
    k_probs_finish(const double* __restrict__ partial, uint64_t nchunks, uint64_t nbins,
                   double* __restrict__ out) {
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= nbins) return;
  Acc acc;
  for (uint64_t c = lane; c < nchunks; c += 32) acc.add(partial[warp * nchunks + c]);
  // Combine lanes: exchange (s, c) pairs and keep compensating.
  double s = acc.s, cc = acc.c;
  for (int o = 16; o > 0; o >>= 1) {
    const double os = __shfl_xor_sync(0xffffffffu, s, o);
    const double oc = __shfl_xor_sync(0xffffffffu, cc, o);
    const double t = s + os;
    double e;
    if (fabs(s) >= fabs(os))
      e = (s - t) + os;
    else
      e = (os - t) + s;
    s = t;
    cc = cc + oc + e;
  }
  if (lane == 0) out[warp] = s + cc;
}

// All single-qubit marginals in one read of the state.  Chunk c holds amplitudes
// [c*8192, (c+1)*8192); thread t of a block visits c*8192 + t + 256*j for j < 32, so
// state bits 0..7 are fixed per thread, bits 8..12 are the bits of j and bits 13.. the
// bits of c.  Blocks stride over chunks.  partial[block*(n+1) + p] = mass with state
// bit p set; partial[block*(n+1) + n] = total mass.
constexpr int MARG_CHUNK_BITS = 13;

template <typename R>
__global__ void __launch_bounds__(QSV_THREADS)
    k_marginals(const CT<R>* __restrict__ psi, int n, uint64_t nchunks, double* __restrict__ partial) {
  using S = Sq<R>;
  __shared__ double sh[32];
  typename S::Accum tot, vj[5], vc[QSV_MAXN - MARG_CHUNK_BITS];
  for (uint64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const CT<R>* base = psi + (c << MARG_CHUNK_BITS) + threadIdx.x;
    typename S::Accum tc;
#pragma unroll
    for (int j0 = 0; j0 < 32; j0 += 8) {
      CT<R> v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u)
        v[u] = QSV_IN_BOUNDS((c << MARG_CHUNK_BITS) + threadIdx.x + ((j0 + u) << 8), nchunks << MARG_CHUNK_BITS)
                   ? base[(j0 + u) << 8]
                   : CT<R>{};
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int j = j0 + u;
        const auto t = S::term(v[u]);
        tc.add(t);
#pragma unroll
        for (int b = 0; b < 5; ++b)
          if ((j >> b) & 1) vj[b].add(t);
      }
    }
    tot.merge(tc);
#pragma unroll
    for (int b = 0; b < QSV_MAXN - MARG_CHUNK_BITS; ++b)
      if (b < n - MARG_CHUNK_BITS && ((c >> b) & 1ull)) vc[b].merge(tc);
  }
  double* row = partial + (uint64_t)blockIdx.x * (n + 1);
  const double t = tot.value();
  double r = block_sum(t, sh);
  if (threadIdx.x == 0) row[n] = r;
  for (int p = 0; p < 8; ++p) {
    r = block_sum(((threadIdx.x >> p) & 1u) ? t : 0.0, sh);
    if (threadIdx.x == 0) row[p] = r;
  }
#pragma unroll
  for (int b = 0; b < 5; ++b) {
    r = block_sum(vj[b].value(), sh);
    if (threadIdx.x == 0) row[8 + b] = r;
  }
#pragma unroll
  for (int b = 0; b < QSV_MAXN - MARG_CHUNK_BITS; ++b) {
    if (b < n - MARG_CHUNK_BITS) {
      r = block_sum(vc[b].value(), sh);
      if (threadIdx.x == 0) row[MARG_CHUNK_BITS + b] = r;
    }
  }
}

// Column sums of partial[nblocks][n+1], one warp per column.
__global__ void __launch_bounds__(QSV_THREADS)
    k_columns_finish(const double* __restrict__ partial, uint64_t nrows, int ncols,
                     double* __restrict__ out) {
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= (uint64_t)ncols) return;
  Acc acc;
  for (uint64_t r = lane; r < nrows; r += 32) acc.add(partial[r * ncols + warp]);
  double s = acc.s, cc = acc.c;
  for (int o = 16; o > 0; o >>= 1) {
    const double os = __shfl_xor_sync(0xffffffffu, s, o);
    const double oc = __shfl_xor_sync(0xffffffffu, cc, o);
    const double t = s + os;
    double e;
    if (fabs(s) >= fabs(os))
      e = (s - t) + os;
    else
      e = (os - t) + s;
    s = t;
    cc = cc + oc + e;
  }
  if (lane == 0) out[warp] = s + cc;
}

// ---- collapse / reduce --------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(QSV_THREADS)
    k_collapse(CT<R>* __restrict__ psi, uint64_t total, uint64_t mask, uint64_t pattern,
               double scale) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += stride) {
    CT<R> v;
    if ((i & mask) == pattern) {
      v = psi[i];
      v.x = R((double)v.x * scale);
      v.y = R((double)v.y * scale);
    } else {
      v.x = R(0);
      v.y = R(0);
    }
    psi[i] = v;
  }
}

struct ReduceArgs {
  uint64_t total_out;
  uint64_t pattern;
  int npos;
  int pos[QSV_MAXQ];
  double scale;
};

template <typename R>
__global__ void __launch_bounds__(QSV_THREADS)
    k_reduce(const CT<R>* __restrict__ src, CT<R>* __restrict__ dst,
             const __grid_constant__ ReduceArgs a) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < a.total_out; j += stride) {
    const uint64_t i = qsv_insert_zeros(j, a.pos, a.npos) | a.pattern;
    if (!QSV_IN_BOUNDS(i, a.total_out << a.npos)) continue;
    CT<R> v = src[i];
    v.x = R((double)v.x * a.scale);
    v.y = R((double)v.y * a.scale);
    dst[j] = v;
  }
}

// ---- function oracle: out[x, y, r] = in[x, y ^ f(x), r] ----------------------------------
struct FuncArgs {
  uint64_t total;
  int n1, n2;
  int p1[QSV_MAXQ];  // reg1 positions, first = MSB of x
  int p2[QSV_MAXQ];  // reg2 positions, first = MSB of y
};

template <typename R>
__global__ void __launch_bounds__(QSV_THREADS)
    k_func(const CT<R>* __restrict__ src, CT<R>* __restrict__ dst,
           const long long* __restrict__ table, const __grid_constant__ FuncArgs a) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < a.total; i += stride) {
    uint64_t x = 0;
    for (int j = 0; j < a.n1; ++j) x = (x << 1) | ((i >> a.p1[j]) & 1ull);
    const uint64_t f = (uint64_t)table[x];
    uint64_t flip = 0;
    for (int j = 0; j < a.n2; ++j)
      if ((f >> (a.n2 - 1 - j)) & 1ull) flip |= 1ull << a.p2[j];
    if (!QSV_IN_BOUNDS(i ^ flip, a.total)) continue;
    dst[i] = src[i ^ flip];
  }
}

// ---- inner product <a|b> over two states (any dtype pair) --------------------------------
template <typename RA, typename RB>
__global__ void __launch_bounds__(QSV_THREADS)
    k_inner_partial(const CT<RA>* __restrict__ a, const CT<RB>* __restrict__ b, uint64_t total,
                    double* __restrict__ partial) {
  __shared__ double sh[32];
  Acc re, im;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += stride) {
    const CT<RA> x = a[i];
    const CT<RB> y = b[i];
    const double xr = x.x, xi = x.y, yr = y.x, yi = y.y;
    re.add(fma(xr, yr, xi * yi));
    im.add(fma(xr, yi, -xi * yr));
  }
  const double r = block_sum(re.value(), sh);
  const double q = block_sum(im.value(), sh);
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x] = r;
    partial[2 * blockIdx.x + 1] = q;
  }
}

}  // namespace

// ======================================================================================
// Host side
// ======================================================================================
namespace {

inline bool is_c64(const qsv_state* s) { return s->dtype == QSV_C64; }

template <typename R>
CT<R> to_ct(const double* c) {
  CT<R> v;
  v.x = R(c[0]);
  v.y = R(c[1]);
  return v;
}

int launch_basis(qsv_state* s, uint64_t index) {
  if (is_c64(s))
    k_set_basis<float><<<1, 1, 0, s->stream>>>((float2*)s->d_amp, index);
  else
    k_set_basis<double><<<1, 1, 0, s->stream>>>((double2*)s->d_amp, index);
  return check_launch(s, "set_basis");
}

// Collects target/control positions and checks they are disjoint.
struct GateGeom {
  int k = 0, nc = 0;
  int tpos[QSV_MAXQ];
  int cpos[QSV_MAXQ];
  int sorted[QSV_MAXQ];
  int npos = 0;
  uint64_t ctrl = 0;
};

int gate_geometry(qsv_state* s, int k, const int* targets, int nc, const int* controls, GateGeom& g) {
  if (k < 0 || nc < 0 || k + nc > QSV_MAXQ || k + nc > s->n)
    return set_error(s, QSV_ERR_INVALID, "bad gate width k=%d controls=%d for n=%d", k, nc, s->n);
  uint64_t seen = 0;
  int rc = to_positions(s, k, targets, g.tpos, &seen);
  if (rc) return rc;
  rc = to_positions(s, nc, controls, g.cpos, &seen);
  if (rc) return rc;
  g.k = k;
  g.nc = nc;
  g.npos = k + nc;
  for (int i = 0; i < k; ++i) g.sorted[i] = g.tpos[i];
  for (int i = 0; i < nc; ++i) {
    g.sorted[k + i] = g.cpos[i];
    g.ctrl |= 1ull << g.cpos[i];
  }
  std::sort(g.sorted, g.sorted + g.npos);
  return QSV_OK;
}

uint64_t target_offset(const GateGeom& g, unsigned j) {
  uint64_t off = 0;
  for (int b = 0; b < g.k; ++b)
    if ((j >> (g.k - 1 - b)) & 1u) off |= 1ull << g.tpos[b];
  return off;
}

template <typename R, int K>
int launch_dense(qsv_state* s, const GateGeom& g, const double* mat) {
  constexpr int D = 1 << K;
  const uint64_t ngroups = 1ull << (s->n - g.k - g.nc);
  if (K == 1 && g.nc == 0) {
    Dense1Args<R> a;
    a.ngroups = ngroups;
    a.p = g.tpos[0];
    a.m00 = to_ct<R>(mat + 0);
    a.m01 = to_ct<R>(mat + 2);
    a.m10 = to_ct<R>(mat + 4);
    a.m11 = to_ct<R>(mat + 6);
    const bool real = mat[1] == 0.0 && mat[3] == 0.0 && mat[5] == 0.0 && mat[7] == 0.0;
    if (real)
      k_dense1<R, true><<<grid_for(s, ngroups), QSV_THREADS, 0, s->stream>>>((CT<R>*)s->d_amp, a);
    else
      k_dense1<R, false><<<grid_for(s, ngroups), QSV_THREADS, 0, s->stream>>>((CT<R>*)s->d_amp, a);
    return check_launch(s, "dense1");
  }
  auto* a = new (std::nothrow) DenseArgs<R, K>();
  if (!a) return set_error(s, QSV_ERR_OOM, "host allocation failed");
  a->ngroups = ngroups;
  a->ctrl = g.ctrl;
  a->npos = g.npos;
  for (int i = 0; i < g.npos; ++i) a->pos[i] = g.sorted[i];
  // complex64 with a target on address bit 0 (and 1): reorder the matrix index so its
  // lowest bits are those address bits (targets by descending position; new index j'
  // reads old index perm[j']) and move 2^VB adjacent amplitudes per access.
  int vb = 0;
  if (std::is_same<R, float>::value && K <= 3 && K >= 1) {
    int order[8];
    for (int b = 0; b < K; ++b) order[b] = b;
    std::sort(order, order + K, [&](int x, int y) { return g.tpos[x] > g.tpos[y]; });
    if (g.tpos[order[K - 1]] == 0) vb = (K >= 2 && g.tpos[order[K - 2]] == 1) ? 2 : 1;
    if (vb) {
      GateGeom gs = g;
      for (int b = 0; b < K; ++b) gs.tpos[b] = g.tpos[order[b]];
      unsigned perm[8];
      for (unsigned jn = 0; jn < (unsigned)D; ++jn) {
        unsigned jo = 0;
        for (int b = 0; b < K; ++b)
          if ((jn >> (K - 1 - b)) & 1u) jo |= 1u << (K - 1 - order[b]);
        perm[jn] = jo;
      }
      for (int j = 0; j < D; ++j) a->off[j] = target_offset(gs, j);
      for (int r = 0; r < D; ++r)
        for (int c = 0; c < D; ++c) a->m[r * D + c] = to_ct<R>(mat + 2 * (perm[r] * D + perm[c]));
    }
  }
  if (!vb) {
    for (int j = 0; j < D; ++j) a->off[j] = target_offset(g, j);
    for (int j = 0; j < D * D; ++j) a->m[j] = to_ct<R>(mat + 2 * j);
  }
  const unsigned grid = grid_for(s, ngroups);
  if constexpr (K <= 3 && std::is_same<R, float>::value) {
    if (vb == 2 && K >= 2)
      k_dense<R, K, (K >= 2 ? 2 : 1)><<<grid, QSV_THREADS, 0, s->stream>>>((CT<R>*)s->d_amp, *a);
    else if (vb == 1)
      k_dense<R, K, 1><<<grid, QSV_THREADS, 0, s->stream>>>((CT<R>*)s->d_amp, *a);
    else
      k_dense<R, K, 0><<<grid, QSV_THREADS, 0, s->stream>>>((CT<R>*)s->d_amp, *a);
  } else {
    k_dense<R, K, 0><<<grid, QSV_THREADS, 0, s->stream>>>((CT<R>*)s->d_amp, *a);
  }
  delete a;
  return check_launch(s, "dense");
}

template <typename R>
int dispatch_dense(qsv_state* s, const GateGeom& g, const double* mat) {
  switch (g.k) {
    case 1: return launch_dense<R, 1>(s, g, mat);
    case 2: return launch_dense<R, 2>(s, g, mat);
    case 3: return launch_dense<R, 3>(s, g, mat);
    case 4: return launch_dense<R, 4>(s, g, mat);
    case 5: return launch_dense<R, 5>(s, g, mat);
    default: return set_error(s, QSV_ERR_UNSUPPORTED, "dense gate on %d targets (max 5)", g.k);
  }
}

template <typename R>
int launch_diag(qsv_state* s, const GateGeom& g, const double* diag) {
  auto* a = new (std::nothrow) DiagArgs<R>();
  if (!a) return set_error(s, QSV_ERR_OOM, "host allocation failed");
  a->ngroups = 1ull << (s->n - g.k - g.nc);
  a->ctrl = g.ctrl;
  a->npos = g.npos;
  for (int i = 0; i < g.npos; ++i) a->pos[i] = g.sorted[i];
  int ne = 0;
  for (unsigned j = 0; j < (1u << g.k); ++j) {
    if (diag[2 * j] == 1.0 && diag[2 * j + 1] == 0.0) continue;
    if (ne >= QSV_MAXDIAG) {
      delete a;
      return set_error(s, QSV_ERR_UNSUPPORTED, "diagonal with more than %d non-unit entries", QSV_MAXDIAG);
    }
    a->off[ne] = target_offset(g, j);
    a->ph[ne] = to_ct<R>(diag + 2 * j);
    ++ne;
  }
  a->nent = ne;
  int rc = QSV_OK;
  if (ne > 0) {
    k_diag<R><<<grid_for(s, a->ngroups), QSV_THREADS, 0, s->stream>>>((CT<R>*)s->d_amp, *a);
    rc = check_launch(s, "diag");
  }
  delete a;
  return rc;
}

template <typename R, int K>
int launch_mono(qsv_state* s, const GateGeom& g, const int* perm, const double* phase) {
  constexpr int D = 1 << K;
  MonoArgs<R, K> a;
  a.ngroups = 1ull << (s->n - g.k - g.nc);
  a.ctrl = g.ctrl;
  a.npos = g.npos;
  for (int i = 0; i < g.npos; ++i) a.pos[i] = g.sorted[i];
  a.exact = 0;
  for (int r = 0; r < D; ++r) {
    if (perm[r] < 0 || perm[r] >= D) return set_error(s, QSV_ERR_INVALID, "permutation entry out of range");
    a.off[r] = target_offset(g, r);
    a.perm[r] = perm[r];
    a.ph[r] = to_ct<R>(phase + 2 * r);
    if (phase[2 * r] == 1.0 && phase[2 * r + 1] == 0.0) a.exact |= 1u << r;
  }
  if (a.exact == (1u << D) - 1u)
    k_mono<R, K, true><<<grid_for(s, a.ngroups), QSV_THREADS, 0, s->stream>>>((CT<R>*)s->d_amp, a);
  else
    k_mono<R, K, false><<<grid_for(s, a.ngroups), QSV_THREADS, 0, s->stream>>>((CT<R>*)s->d_amp, a);
  return check_launch(s, "monomial");
}

template <typename R>
int dispatch_mono(qsv_state* s, const GateGeom& g, const int* perm, const double* phase) {
  switch (g.k) {
    case 1: return launch_mono<R, 1>(s, g, perm, phase);
    case 2: return launch_mono<R, 2>(s, g, perm, phase);
    case 3: return launch_mono<R, 3>(s, g, perm, phase);
    default: return set_error(s, QSV_ERR_UNSUPPORTED, "monomial gate on %d targets (max 3)", g.k);
  }
}

template <typename R>
int launch_probs(qsv_state* s, int m, const int* pos_in_order, double* d_out_or_null,
                 double* host_out) {
  // pos_in_order[j] = bit position of outcome bit j.
  ProbArgs a;
  a.m = m;
  a.npos = m;
  uint64_t nbins = 1ull << m;
  a.nbins = nbins;
  a.nrest = 1ull << (s->n - m);
  for (int j = 0; j < m; ++j) {
    a.binbit[j] = 1ull << pos_in_order[j];
    a.pos[j] = pos_in_order[j];
  }
  std::sort(a.pos, a.pos + m);
  const uint64_t target_blocks = (uint64_t)std::max(1, s->sm_count) * 32;
  int rc;
  if (nbins > 65535ull * 8 || (a.nrest < 4096 && nbins >= 4096)) {
    // Many outcomes, short sums: one thread per outcome.
    rc = ensure_scratch(s, nbins * sizeof(double));
    if (rc) return rc;
    double* out = (double*)s->d_scratch;
    a.chunk = a.nrest;
    a.nchunks = 1;
    const unsigned blocks = (unsigned)((nbins + QSV_THREADS - 1) / QSV_THREADS);
    k_probs_perbin<R><<<blocks, QSV_THREADS, 0, s->stream>>>((const CT<R>*)s->d_amp, a, out);
    rc = check_launch(s, "probs_perbin");
    if (rc) return rc;
    QSV_CUDA(s, cudaMemcpyAsync(host_out, out, nbins * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    QSV_CUDA(s, cudaStreamSynchronize(s->stream));
    return QSV_OK;
  }
  uint64_t chunk = 4096;
  while (chunk < a.nrest && nbins * ((a.nrest + chunk - 1) / chunk) > target_blocks) chunk <<= 1;
  if (chunk > a.nrest) chunk = a.nrest;
  a.chunk = chunk;
  a.nchunks = (a.nrest + chunk - 1) / chunk;
  const uint64_t nblk = nbins * a.nchunks;
  rc = ensure_scratch(s, (nblk + nbins) * sizeof(double));
  if (rc) return rc;
  double* partial = (double*)s->d_scratch;
  double* out = partial + nblk;
  dim3 grid;
  grid.x = (unsigned)std::min<uint64_t>(nblk, 65535ull * 1024);
  grid.y = (unsigned)((nblk + grid.x - 1) / grid.x);
  k_probs_partial<R><<<grid, QSV_THREADS, 0, s->stream>>>((const CT<R>*)s->d_amp, a, partial);
  rc = check_launch(s, "probs_partial");
  if (rc) return rc;
  const unsigned fblocks = (unsigned)((nbins * 32 + QSV_THREADS - 1) / QSV_THREADS);
  k_probs_finish<<<fblocks, QSV_THREADS, 0, s->stream>>>(partial, a.nchunks, nbins, out);
  rc = check_launch(s, "probs_finish");
  if (rc) return rc;
  (void)d_out_or_null;
  QSV_CUDA(s, cudaMemcpyAsync(host_out, out, nbins * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  QSV_CUDA(s, cudaStreamSynchronize(s->stream));
  return QSV_OK;
}

}  // namespace

namespace {
constexpr size_t kStageMinBytes = size_t(32) << 20;  // reads below this go straight to the caller
constexpr size_t kStageChunk = size_t(64) << 20;     // two pinned halves of this size per handle

// memcpy split over a few host threads (host memory bandwidth needs several cores).
void parallel_copy(char* dst, const char* src, size_t len) {
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const unsigned nt = std::min<unsigned>(16, hw);
  if (nt <= 1 || len < (size_t(4) << 20)) {
    memcpy(dst, src, len);
    return;
  }
  std::vector<std::thread> pool;
  const size_t slice = (len + nt - 1) / nt;
  for (unsigned t = 1; t < nt; ++t) {
    const size_t off = t * slice;
    if (off >= len) break;
    pool.emplace_back([=] { memcpy(dst + off, src + off, std::min(slice, len - off)); });
  }
  memcpy(dst, src, std::min(slice, len));
  for (auto& th : pool) th.join();
}

// Writes one byte per 4 KiB page of [p, p+len) from several threads so the kernel maps
// the pages in parallel; the bytes are overwritten by the copy that follows.
void parallel_touch(char* p, size_t len) {
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const unsigned nt = std::min<unsigned>(16, hw);
  auto touch = [](char* a, size_t n) {
    for (size_t i = 0; i < n; i += 4096) reinterpret_cast<volatile char*>(a)[i] = 0;
  };
  if (nt <= 1) {
    touch(p, len);
    return;
  }
  std::vector<std::thread> pool;
  const size_t slice = ((len + nt - 1) / nt + 4095) & ~size_t(4095);
  for (unsigned t = 1; t < nt; ++t) {
    const size_t off = t * slice;
    if (off >= len) break;
    pool.emplace_back([=] { touch(p + off, std::min(slice, len - off)); });
  }
  touch(p, std::min(slice, len));
  for (auto& th : pool) th.join();
}
}  // namespace

// ======================================================================================
// C ABI
// ======================================================================================
extern "C" {

const char* qsv_status_string(int status) {
  switch (status) {
    case QSV_OK: return "ok";
    case QSV_ERR_INVALID: return "invalid argument";
    case QSV_ERR_OOM: return "out of device memory";
    case QSV_ERR_CUDA: return "CUDA error";
    case QSV_ERR_TIMEOUT: return "device wait timed out";
    case QSV_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
  }
}

const char* qsv_last_error(const qsv_state* s) { return s ? s->err : g_global_err; }

unsigned long long qsv_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

// ---- resources of destroyed states, parked for the next state ----------------------------
// A caller that runs one circuit per state (create, apply, read, destroy in a loop) would
// otherwise map a 2^n buffer, page-lock image slots and unmap both for every circuit.
// qsv_destroy parks a state's buffers (at most kMaxSpares states' worth, amplitude buffers
// up to kMaxParkedAmp bytes in total, so other allocators in the process keep the HBM of
// large states); qsv_create takes them back: the
// amplitude buffer when device and size match, the other buffers when the device
// matches.  A failed amplitude allocation releases the parked buffers and retries;
// qsv_trim releases them on request.
namespace {
struct Spare {
  int device = -1;
  void* d_amp = nullptr;
  size_t amp_bytes = 0;
  int* d_flag = nullptr;
  void* d_scratch = nullptr;
  size_t scratch_bytes = 0;
  void* d_images = nullptr;
  size_t d_images_bytes = 0;
  void* h_img[qsv_state::kImageSlots] = {nullptr};
  size_t h_img_bytes[qsv_state::kImageSlots] = {0};
  cudaEvent_t img_ev[qsv_state::kImageSlots] = {nullptr};
  void* h_stage = nullptr;
  size_t h_stage_bytes = 0;
  cudaStream_t stream = nullptr;
};
constexpr size_t kMaxSpares = 2;
constexpr size_t kMaxParkedAmp = size_t(8) << 30;
std::mutex g_spare_mu;
std::vector<Spare> g_spares;

void free_spare(Spare& sp, bool keep_amp = false) {
  if (sp.d_amp && !keep_amp) cudaFree(sp.d_amp);
  if (sp.d_flag) cudaFree(sp.d_flag);
  if (sp.d_scratch) cudaFree(sp.d_scratch);
  if (sp.d_images) cudaFree(sp.d_images);
  for (int i = 0; i < qsv_state::kImageSlots; ++i) {
    if (sp.h_img[i]) cudaFreeHost(sp.h_img[i]);
    if (sp.img_ev[i]) cudaEventDestroy(sp.img_ev[i]);
  }
  if (sp.h_stage) cudaFreeHost(sp.h_stage);
  if (sp.stream) cudaStreamDestroy(sp.stream);
  sp = Spare{};
}

// Moves a parked state's resources into s (same device; the amplitude buffer only if
// its size is `bytes`).  Returns false if nothing was parked for this device.
bool take_spare(qsv_state* s, size_t bytes) {
  Spare sp;
  {
    std::lock_guard<std::mutex> lk(g_spare_mu);
    int pick = -1;
    for (size_t i = 0; i < g_spares.size(); ++i)
      if (g_spares[i].device == s->device && (pick < 0 || g_spares[i].amp_bytes == bytes)) pick = (int)i;
    if (pick < 0) return false;
    sp = g_spares[(size_t)pick];
    g_spares.erase(g_spares.begin() + pick);
  }
  if (sp.d_amp && sp.amp_bytes != bytes) {
    cudaFree(sp.d_amp);
    sp.d_amp = nullptr;
  }
  s->d_amp = sp.d_amp;
  s->d_flag = sp.d_flag;
  s->d_scratch = sp.d_scratch;
  s->scratch_bytes = sp.scratch_bytes;
  s->d_images = sp.d_images;
  s->d_images_bytes = sp.d_images_bytes;
  for (int i = 0; i < qsv_state::kImageSlots; ++i) {
    s->h_img[i] = sp.h_img[i];
    s->h_img_bytes[i] = sp.h_img_bytes[i];
    s->img_ev[i] = sp.img_ev[i];
  }
  s->h_stage = sp.h_stage;
  s->h_stage_bytes = sp.h_stage_bytes;
  s->own_stream = sp.stream;
  return true;
}

// Parks s's resources (s's stream is idle).  Returns false if the cache is full.
bool park(qsv_state* s) {
  std::lock_guard<std::mutex> lk(g_spare_mu);
  if (g_spares.size() >= kMaxSpares) return false;
  size_t amp_total = s->d_amp ? (size_t(1) << s->n) * s->amp_bytes : 0;
  for (const Spare& sp : g_spares)
    if (sp.device == s->device) amp_total += sp.amp_bytes;
  Spare sp;
  sp.device = s->device;
  if (s->d_amp && amp_total <= kMaxParkedAmp) {
    sp.d_amp = s->d_amp;
    sp.amp_bytes = (size_t(1) << s->n) * s->amp_bytes;
  } else if (s->d_amp) {
    cudaFree(s->d_amp);
  }
  sp.d_flag = s->d_flag;
  sp.d_scratch = s->d_scratch;
  sp.scratch_bytes = s->scratch_bytes;
  sp.d_images = s->d_images;
  sp.d_images_bytes = s->d_images_bytes;
  for (int i = 0; i < qsv_state::kImageSlots; ++i) {
    sp.h_img[i] = s->h_img[i];
    sp.h_img_bytes[i] = s->h_img_bytes[i];
    sp.img_ev[i] = s->img_ev[i];
  }
  sp.h_stage = s->h_stage;
  sp.h_stage_bytes = s->h_stage_bytes;
  sp.stream = s->own_stream;
  g_spares.push_back(sp);
  return true;
}

void release_spares(int device) {
  std::vector<Spare> drop;
  {
    std::lock_guard<std::mutex> lk(g_spare_mu);
    for (size_t i = 0; i < g_spares.size();) {
      if (device < 0 || g_spares[i].device == device) {
        drop.push_back(g_spares[i]);
        g_spares.erase(g_spares.begin() + (long)i);
      } else {
        ++i;
      }
    }
  }
  for (Spare& sp : drop) free_spare(sp);
}
}  // namespace

}  // extern "C"

namespace qsv {
int oob_take_core(unsigned long long* count, unsigned long long* first) {
#ifdef QSV_BOUNDS_CHECK
  return qsv_oob_take_unit(count, first);
#else
  (void)count;
  (void)first;
  return 0;
#endif
}
}  // namespace qsv

extern "C" {

int qsv_bounds_report(unsigned long long* count, unsigned long long* first_index) {
  if (!count || !first_index) return set_error(nullptr, QSV_ERR_INVALID, "null output");
  *count = 0;
  *first_index = 0;
#ifdef QSV_BOUNDS_CHECK
  cudaDeviceSynchronize();
  if (oob_take_core(count, first_index) || oob_take_fused(count, first_index) ||
      oob_take_adjoint(count, first_index) || oob_take_circuits(count, first_index) ||
      oob_take_adjtc(count, first_index))
    return set_error(nullptr, QSV_ERR_CUDA, "reading the bounds words failed");
  return QSV_OK;
#else
  return set_error(nullptr, QSV_ERR_UNSUPPORTED, "not a bounds-checked build (libqsv_checked.so)");
#endif
}

int qsv_trim(void) {
  release_spares(-1);
  return QSV_OK;
}

int qsv_create(int n, int dtype, qsv_state** out) {
  if (!out) return set_error(nullptr, QSV_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (n < 1 || n > QSV_MAXN) return set_error(nullptr, QSV_ERR_INVALID, "n=%d outside [1, %d]", n, QSV_MAXN);
  if (dtype != QSV_C64 && dtype != QSV_C128) return set_error(nullptr, QSV_ERR_INVALID, "unknown dtype %d", dtype);
  // Host-side fault injection: a failed state allocation, before any device call.
  if (const char* f = getenv("QSV_INJECT_ALLOC_FAILURE"))
    if (f[0] && f[0] != '0')
      return set_error(nullptr, QSV_ERR_OOM, "state allocation of %zu bytes failed (injected)",
                       ((size_t)1 << n) * (dtype == QSV_C64 ? 8 : 16));
  auto* s = new (std::nothrow) qsv_state();
  if (!s) return set_error(nullptr, QSV_ERR_OOM, "host allocation failed");
  s->n = n;
  s->dtype = dtype;
  s->amp_bytes = dtype == QSV_C64 ? 8 : 16;
  const size_t bytes = (size_t(1) << n) * s->amp_bytes;
  cudaError_t e = cudaGetDevice(&s->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, s->device);
  if (e == cudaSuccess) take_spare(s, bytes);
  if (e == cudaSuccess && !s->own_stream) e = cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    qsv_destroy(s);
    return set_error(nullptr, QSV_ERR_CUDA, "device setup: %s", cudaGetErrorString(e));
  }
  s->stream = s->own_stream;
  if (!s->d_amp && cudaMalloc(&s->d_amp, bytes) != cudaSuccess) {
    // Parked buffers of other states may hold the memory: release them and retry.
    cudaGetLastError();
    s->d_amp = nullptr;
    release_spares(s->device);
    if (cudaMalloc(&s->d_amp, bytes) != cudaSuccess) s->d_amp = nullptr;
  }
  if (s->d_amp && !s->d_flag && cudaMalloc(&s->d_flag, sizeof(int)) != cudaSuccess) s->d_flag = nullptr;
  if (!s->d_amp || !s->d_flag) {
    cudaGetLastError();
    s->n = 0;  // nothing to park: qsv_destroy frees what was taken
    qsv_destroy(s);
    return set_error(nullptr, QSV_ERR_OOM, "device allocation of %zu bytes failed", bytes);
  }
  int rc = QSV_OK;
  if (cudaMemsetAsync(s->d_amp, 0, bytes, s->stream) != cudaSuccess ||
      cudaMemsetAsync(s->d_flag, 0, sizeof(int), s->stream) != cudaSuccess)
    rc = set_error(nullptr, QSV_ERR_CUDA, "memset failed");
  if (!rc) rc = launch_basis(s, 0);
  if (rc) {
    if (!s->err[0]) set_error(nullptr, rc, "initialisation failed");
    else set_error(nullptr, rc, "%s", s->err);
    qsv_destroy(s);
    return rc;
  }
  *out = s;
  return QSV_OK;
}

int qsv_destroy(qsv_state* s) {
  if (!s) return QSV_OK;
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->own_stream && s->own_stream != s->stream) cudaStreamSynchronize(s->own_stream);
  // A healthy state's buffers are parked for the next state; otherwise freed.
  bool healthy = s->n > 0 && s->d_amp && s->d_flag && cudaGetLastError() == cudaSuccess;
  if (healthy && s->d_flag) {
    int flag = 0;
    healthy = cudaMemcpy(&flag, s->d_flag, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess && flag == 0;
  }
  if (healthy && park(s)) {
    delete s;
    return QSV_OK;
  }
  if (s->d_amp) cudaFree(s->d_amp);
  if (s->d_flag) cudaFree(s->d_flag);
  if (s->d_scratch) cudaFree(s->d_scratch);
  if (s->d_images) cudaFree(s->d_images);
  for (int i = 0; i < qsv_state::kImageSlots; ++i) {
    if (s->h_img[i]) cudaFreeHost(s->h_img[i]);
    if (s->img_ev[i]) cudaEventDestroy(s->img_ev[i]);
  }
  if (s->h_stage) cudaFreeHost(s->h_stage);
  if (s->own_stream) cudaStreamDestroy(s->own_stream);
  delete s;
  return QSV_OK;
}

int qsv_set_stream(qsv_state* s, void* stream) {
  QSV_CHECK_HANDLE(s);
  QSV_CUDA(s, cudaStreamSynchronize(s->stream));
  s->stream = stream ? (cudaStream_t)stream : s->own_stream;
  return QSV_OK;
}

int qsv_synchronize(qsv_state* s) {
  QSV_CHECK_HANDLE(s);
  QSV_CUDA(s, cudaStreamSynchronize(s->stream));
  int flag = 0;
  QSV_CUDA(s, cudaMemcpy(&flag, s->d_flag, sizeof(int), cudaMemcpyDeviceToHost));
  if (flag) {
    cudaMemset(s->d_flag, 0, sizeof(int));
    return set_error(s, QSV_ERR_TIMEOUT, "a bounded device wait gave up (code %d)", flag);
  }
  return QSV_OK;
}

int qsv_num_qubits(const qsv_state* s) { return s ? s->n : -1; }
int qsv_dtype(const qsv_state* s) { return s ? s->dtype : -1; }
void* qsv_device_ptr(qsv_state* s) { return s ? s->d_amp : nullptr; }

int qsv_set_product_state(qsv_state* s, int ngroups, const int* group_sizes, const int* qubits_flat,
                          const double* feeds_c128) {
  QSV_CHECK_HANDLE(s);
  const uint64_t total = 1ull << s->n;
  if (ngroups == 0) {
    QSV_CUDA(s, cudaMemsetAsync(s->d_amp, 0, total * s->amp_bytes, s->stream));
    return launch_basis(s, 0);
  }
  if (ngroups < 0 || ngroups > QSV_MAXQ || !group_sizes || !qubits_flat || !feeds_c128)
    return set_error(s, QSV_ERR_INVALID, "bad feed description");
  ProductArgs a;
  a.total = total;
  a.ngroups = ngroups;
  uint64_t seen = 0;
  int q = 0;
  uint64_t nfeed = 0;
  for (int g = 0; g < ngroups; ++g) {
    const int sz = group_sizes[g];
    if (sz < 1 || q + sz > s->n) return set_error(s, QSV_ERR_INVALID, "feed group %d has bad size %d", g, sz);
    int rc = to_positions(s, sz, qubits_flat + q, a.pos + q, &seen);
    if (rc) return rc;
    a.size[g] = sz;
    a.feed_off[g] = nfeed;
    nfeed += 1ull << sz;
    q += sz;
  }
  a.nq = q;
  a.unfed_mask = ((s->n == 64) ? ~0ull : ((1ull << s->n) - 1ull)) & ~seen;
  int rc = ensure_scratch(s, nfeed * sizeof(double2));
  if (rc) return rc;
  QSV_CUDA(s, cudaMemcpyAsync(s->d_scratch, feeds_c128, nfeed * sizeof(double2), cudaMemcpyHostToDevice, s->stream));
  const unsigned grid = grid_for(s, total);
  if (is_c64(s))
    k_product<float><<<grid, QSV_THREADS, 0, s->stream>>>((float2*)s->d_amp, (const double2*)s->d_scratch, a);
  else
    k_product<double><<<grid, QSV_THREADS, 0, s->stream>>>((double2*)s->d_amp, (const double2*)s->d_scratch, a);
  return check_launch(s, "product_state");
}

int qsv_write_range(qsv_state* s, const void* host, uint64_t start, uint64_t count) {
  QSV_CHECK_HANDLE(s);
  if (start + count > (1ull << s->n) || (count && !host))
    return set_error(s, QSV_ERR_INVALID, "range [%llu, +%llu) outside the state", (unsigned long long)start,
                     (unsigned long long)count);
  if (!count) return QSV_OK;
  QSV_CUDA(s, cudaMemcpyAsync((char*)s->d_amp + start * s->amp_bytes, host, count * s->amp_bytes,
                              cudaMemcpyHostToDevice, s->stream));
  return QSV_OK;
}

int qsv_add_range(qsv_state* s, const void* host, uint64_t start, uint64_t count) {
  QSV_CHECK_HANDLE(s);
  if (start + count > (1ull << s->n) || (count && !host))
    return set_error(s, QSV_ERR_INVALID, "range outside the state");
  if (!count) return QSV_OK;
  int rc = ensure_scratch(s, count * s->amp_bytes);
  if (rc) return rc;
  QSV_CUDA(s, cudaMemcpyAsync(s->d_scratch, host, count * s->amp_bytes, cudaMemcpyHostToDevice, s->stream));
  const unsigned grid = grid_for(s, count);
  if (is_c64(s))
    k_add_range<float><<<grid, QSV_THREADS, 0, s->stream>>>((float2*)s->d_amp + start, (const float2*)s->d_scratch, count);
  else
    k_add_range<double><<<grid, QSV_THREADS, 0, s->stream>>>((double2*)s->d_amp + start, (const double2*)s->d_scratch, count);
  return check_launch(s, "add_range");
}

namespace {
bool is_pinned(const void* p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost;
}
}  // namespace

int qsv_trace_push(const char* name) {
  nvtxRangePushA(name ? name : "");
  return QSV_OK;
}

int qsv_trace_pop(void) {
  nvtxRangePop();
  return QSV_OK;
}

int qsv_host_alloc(uint64_t bytes, void** out) {
  if (!out || bytes == 0) return set_error(nullptr, QSV_ERR_INVALID, "bad host allocation request");
  *out = nullptr;
  if (cudaHostAlloc(out, bytes, cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    *out = nullptr;
    return set_error(nullptr, QSV_ERR_OOM, "page-locked host allocation of %llu bytes failed",
                     (unsigned long long)bytes);
  }
  return QSV_OK;
}

int qsv_host_free(void* p) {
  if (p && cudaFreeHost(p) != cudaSuccess) return set_error(nullptr, QSV_ERR_CUDA, "cudaFreeHost failed");
  return QSV_OK;
}

int qsv_read_range(qsv_state* s, void* host, uint64_t start, uint64_t count) {
  QSV_CHECK_HANDLE(s);
  if (start + count > (1ull << s->n) || (count && !host))
    return set_error(s, QSV_ERR_INVALID, "range outside the state");
  if (!count) return QSV_OK;
  const size_t bytes = count * s->amp_bytes;
  const char* src = (const char*)s->d_amp + start * s->amp_bytes;
  if (bytes < kStageMinBytes || is_pinned(host)) {
    // Small reads, and page-locked destinations (qsv_host_alloc): one direct DMA.
    QSV_CUDA(s, cudaMemcpyAsync(host, src, bytes, cudaMemcpyDeviceToHost, s->stream));
    QSV_CUDA(s, cudaStreamSynchronize(s->stream));
    return QSV_OK;
  }
  // Large reads: DMA into two pinned staging halves while host threads copy the
  // previous chunk into the (pageable) destination.
  if (!s->h_stage) {
    if (cudaMallocHost(&s->h_stage, 2 * kStageChunk) != cudaSuccess) {
      cudaGetLastError();
      s->h_stage = nullptr;
      QSV_CUDA(s, cudaMemcpyAsync(host, src, bytes, cudaMemcpyDeviceToHost, s->stream));
      QSV_CUDA(s, cudaStreamSynchronize(s->stream));
      return QSV_OK;
    }
    s->h_stage_bytes = 2 * kStageChunk;
  }
  cudaEvent_t ev[2];
  QSV_CUDA(s, cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming));
  QSV_CUDA(s, cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming));
  char* dst = static_cast<char*>(host);
  // Fault in the destination's pages from several threads while queued kernels still
  // run (first touch of fresh host memory costs about as much as the copy itself).
  parallel_touch(dst, bytes);
  char* stage = static_cast<char*>(s->h_stage);
  const size_t nchunks = (bytes + kStageChunk - 1) / kStageChunk;
  int rc = QSV_OK;
  for (size_t i = 0; i <= nchunks && rc == QSV_OK; ++i) {
    if (i < nchunks) {
      const size_t off = i * kStageChunk, len = std::min(kStageChunk, bytes - off);
      cudaError_t e = cudaMemcpyAsync(stage + (i & 1) * kStageChunk, src + off, len, cudaMemcpyDeviceToHost, s->stream);
      if (e == cudaSuccess) e = cudaEventRecord(ev[i & 1], s->stream);
      if (e != cudaSuccess) rc = set_error(s, QSV_ERR_CUDA, "staged read: %s", cudaGetErrorString(e));
    }
    if (i > 0 && rc == QSV_OK) {
      const size_t j = i - 1, off = j * kStageChunk, len = std::min(kStageChunk, bytes - off);
      cudaError_t e = cudaEventSynchronize(ev[j & 1]);
      if (e != cudaSuccess) {
        rc = set_error(s, QSV_ERR_CUDA, "staged read: %s", cudaGetErrorString(e));
        break;
      }
      parallel_copy(dst + off, stage + (j & 1) * kStageChunk, len);
    }
  }
  if (rc) cudaStreamSynchronize(s->stream);
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  return rc;
}

int qsv_apply_matrix(qsv_state* s, int k, const int* targets, int ncontrols, const int* controls,
                     const double* mat_c128) {
  QSV_CHECK_HANDLE(s);
  if (!mat_c128) return set_error(s, QSV_ERR_INVALID, "null matrix");
  if (k < 1) return set_error(s, QSV_ERR_INVALID, "matrix gate needs at least one target");
  GateGeom g;
  int rc = gate_geometry(s, k, targets, ncontrols, controls, g);
  if (rc) return rc;
  return is_c64(s) ? dispatch_dense<float>(s, g, mat_c128) : dispatch_dense<double>(s, g, mat_c128);
}

int qsv_apply_diagonal(qsv_state* s, int k, const int* targets, int ncontrols, const int* controls,
                       const double* diag_c128) {
  QSV_CHECK_HANDLE(s);
  if (!diag_c128) return set_error(s, QSV_ERR_INVALID, "null diagonal");
  if (k > 10) return set_error(s, QSV_ERR_UNSUPPORTED, "diagonal on %d targets (max 10)", k);
  GateGeom g;
  int rc = gate_geometry(s, k, targets, ncontrols, controls, g);
  if (rc) return rc;
  return is_c64(s) ? launch_diag<float>(s, g, diag_c128) : launch_diag<double>(s, g, diag_c128);
}

int qsv_apply_monomial(qsv_state* s, int k, const int* targets, int ncontrols, const int* controls,
                       const int* perm, const double* phase_c128) {
  QSV_CHECK_HANDLE(s);
  if (!perm || !phase_c128) return set_error(s, QSV_ERR_INVALID, "null permutation");
  GateGeom g;
  int rc = gate_geometry(s, k, targets, ncontrols, controls, g);
  if (rc) return rc;
  return is_c64(s) ? dispatch_mono<float>(s, g, perm, phase_c128) : dispatch_mono<double>(s, g, perm, phase_c128);
}

int qsv_apply_swap(qsv_state* s, int m, const int* a, const int* b, int ncontrols, const int* controls) {
  QSV_CHECK_HANDLE(s);
  if (m < 1 || 2 * m + ncontrols > QSV_MAXQ || 2 * m + ncontrols > s->n)
    return set_error(s, QSV_ERR_INVALID, "bad swap width %d", m);
  SwapArgs args;
  uint64_t seen = 0;
  int rc = to_positions(s, m, a, args.apos, &seen);
  if (!rc) rc = to_positions(s, m, b, args.bpos, &seen);
  if (!rc) rc = to_positions(s, ncontrols, controls, args.cpos, &seen);
  if (rc) return rc;
  if (m == 1) {
    Swap1Args a1;
    a1.npos = 2 + ncontrols;
    a1.pos[0] = args.apos[0];
    a1.pos[1] = args.bpos[0];
    a1.ctrl = 1ull << args.apos[0];
    for (int i = 0; i < ncontrols; ++i) {
      a1.pos[2 + i] = args.cpos[i];
      a1.ctrl |= 1ull << args.cpos[i];
    }
    std::sort(a1.pos, a1.pos + a1.npos);
    a1.flip = (1ull << args.apos[0]) | (1ull << args.bpos[0]);
    a1.nitems = 1ull << (s->n - a1.npos);
    const unsigned grid1 = grid_for(s, (a1.nitems + 1) / 2);
    if (is_c64(s))
      k_swap1<float><<<grid1, QSV_THREADS, 0, s->stream>>>((float2*)s->d_amp, a1);
    else
      k_swap1<double><<<grid1, QSV_THREADS, 0, s->stream>>>((double2*)s->d_amp, a1);
    return check_launch(s, "swap1");
  }
  args.m = m;
  args.ncp = ncontrols;
  args.ctrl = 0;
  for (int i = 0; i < ncontrols; ++i) args.ctrl |= 1ull << args.cpos[i];
  std::sort(args.cpos, args.cpos + ncontrols);
  args.nitems = 1ull << (s->n - ncontrols);
  const unsigned grid = grid_for(s, args.nitems);
  if (is_c64(s))
    k_swap<float><<<grid, QSV_THREADS, 0, s->stream>>>((float2*)s->d_amp, args);
  else
    k_swap<double><<<grid, QSV_THREADS, 0, s->stream>>>((double2*)s->d_amp, args);
  return check_launch(s, "swap");
}

int qsv_probabilities(qsv_state* s, int m, const int* qubits, double* out) {
  QSV_CHECK_HANDLE(s);
  if (!out) return set_error(s, QSV_ERR_INVALID, "null output");
  if (m < 0 || m > s->n || m > 30) return set_error(s, QSV_ERR_INVALID, "bad measured count %d", m);
  int pos[QSV_MAXQ];
  uint64_t seen = 0;
  int rc = to_positions(s, m, qubits, pos, &seen);
  if (rc) return rc;
  return is_c64(s) ? launch_probs<float>(s, m, pos, nullptr, out) : launch_probs<double>(s, m, pos, nullptr, out);
}

int qsv_norm2(qsv_state* s, double* out) { return qsv_probabilities(s, 0, nullptr, out); }

int qsv_qubit_marginals(qsv_state* s, double* out, double* norm2) {
  QSV_CHECK_HANDLE(s);
  if (!out) return set_error(s, QSV_ERR_INVALID, "null output");
  const int n = s->n;
  if (n < 14) {
    // Small states: per-qubit marginal calls.
    double p[2];
    double tot = 0.0;
    for (int q = 0; q < n; ++q) {
      int rc = qsv_probabilities(s, 1, &q, p);
      if (rc) return rc;
      out[q] = p[1];
      tot = p[0] + p[1];
    }
    if (norm2) *norm2 = tot;
    return QSV_OK;
  }
  const uint64_t nchunks = 1ull << (n - MARG_CHUNK_BITS);
  const uint64_t nblocks = std::min<uint64_t>(nchunks, (uint64_t)std::max(1, s->sm_count) * 4);
  const size_t bytes = (nblocks * (n + 1) + (n + 1)) * sizeof(double);
  int rc = ensure_scratch(s, bytes);
  if (rc) return rc;
  double* partial = (double*)s->d_scratch;
  double* col = partial + nblocks * (n + 1);
  if (is_c64(s))
    k_marginals<float><<<(unsigned)nblocks, QSV_THREADS, 0, s->stream>>>((const float2*)s->d_amp, n, nchunks, partial);
  else
    k_marginals<double><<<(unsigned)nblocks, QSV_THREADS, 0, s->stream>>>((const double2*)s->d_amp, n, nchunks, partial);
  rc = check_launch(s, "marginals");
  if (rc) return rc;
  const unsigned fblocks = (unsigned)(((n + 1) * 32 + QSV_THREADS - 1) / QSV_THREADS);
  k_columns_finish<<<fblocks, QSV_THREADS, 0, s->stream>>>(partial, nblocks, n + 1, col);
  rc = check_launch(s, "marginals_finish");
  if (rc) return rc;
  double hostcol[QSV_MAXN + 1];
  QSV_CUDA(s, cudaMemcpyAsync(hostcol, col, (n + 1) * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  QSV_CUDA(s, cudaStreamSynchronize(s->stream));
  // Column p holds the mass with state bit p set; qubit q sits at bit n-1-q.
  for (int q = 0; q < n; ++q) out[q] = hostcol[n - 1 - q];
  if (norm2) *norm2 = hostcol[n];
  return QSV_OK;
}

int qsv_collapse(qsv_state* s, int m, const int* qubits, uint64_t value, double scale) {
  QSV_CHECK_HANDLE(s);
  if (m < 0 || m > s->n) return set_error(s, QSV_ERR_INVALID, "bad measured count %d", m);
  if (m < 64 && value >= (1ull << m)) return set_error(s, QSV_ERR_INVALID, "outcome %llu out of range", (unsigned long long)value);
  int pos[QSV_MAXQ];
  uint64_t seen = 0;
  int rc = to_positions(s, m, qubits, pos, &seen);
  if (rc) return rc;
  uint64_t pattern = 0;
  for (int j = 0; j < m; ++j)
    if ((value >> j) & 1ull) pattern |= 1ull << pos[j];
  const uint64_t total = 1ull << s->n;
  const unsigned grid = grid_for(s, total);
  if (is_c64(s))
    k_collapse<float><<<grid, QSV_THREADS, 0, s->stream>>>((float2*)s->d_amp, total, seen, pattern, scale);
  else
    k_collapse<double><<<grid, QSV_THREADS, 0, s->stream>>>((double2*)s->d_amp, total, seen, pattern, scale);
  return check_launch(s, "collapse");
}

int qsv_reduce(qsv_state* s, int m, const int* qubits, uint64_t value, double scale) {
  QSV_CHECK_HANDLE(s);
  if (m < 1 || m >= s->n) return set_error(s, QSV_ERR_INVALID, "reduce needs 1 <= m < n (m=%d)", m);
  if (value >= (1ull << m)) return set_error(s, QSV_ERR_INVALID, "outcome out of range");
  ReduceArgs a;
  uint64_t seen = 0;
  int pos[QSV_MAXQ];
  int rc = to_positions(s, m, qubits, pos, &seen);
  if (rc) return rc;
  a.pattern = 0;
  for (int j = 0; j < m; ++j) {
    if ((value >> j) & 1ull) a.pattern |= 1ull << pos[j];
    a.pos[j] = pos[j];
  }
  std::sort(a.pos, a.pos + m);
  a.npos = m;
  a.scale = scale;
  a.total_out = 1ull << (s->n - m);
  void* dst = nullptr;
  if (cudaMalloc(&dst, a.total_out * s->amp_bytes) != cudaSuccess) {
    cudaGetLastError();
    return set_error(s, QSV_ERR_OOM, "reduce: allocation failed");
  }
  const unsigned grid = grid_for(s, a.total_out);
  if (is_c64(s))
    k_reduce<float><<<grid, QSV_THREADS, 0, s->stream>>>((const float2*)s->d_amp, (float2*)dst, a);
  else
    k_reduce<double><<<grid, QSV_THREADS, 0, s->stream>>>((const double2*)s->d_amp, (double2*)dst, a);
  rc = check_launch(s, "reduce");
  if (rc) {
    cudaFree(dst);
    return rc;
  }
  QSV_CUDA(s, cudaStreamSynchronize(s->stream));
  cudaFree(s->d_amp);
  s->d_amp = dst;
  s->n -= m;
  return QSV_OK;
}

int qsv_func_apply(qsv_state* s, int n1, const int* reg1, int n2, const int* reg2, const int64_t* table) {
  QSV_CHECK_HANDLE(s);
  if (n1 < 1 || n2 < 1 || n1 + n2 > s->n || n1 > 30 || !table)
    return set_error(s, QSV_ERR_INVALID, "bad register sizes %d, %d", n1, n2);
  FuncArgs a;
  uint64_t seen = 0;
  int rc = to_positions(s, n1, reg1, a.p1, &seen);
  if (!rc) rc = to_positions(s, n2, reg2, a.p2, &seen);
  if (rc) return rc;
  a.n1 = n1;
  a.n2 = n2;
  a.total = 1ull << s->n;
  const size_t tbytes = (size_t(1) << n1) * sizeof(int64_t);
  rc = ensure_scratch(s, tbytes);
  if (rc) return rc;
  QSV_CUDA(s, cudaMemcpyAsync(s->d_scratch, table, tbytes, cudaMemcpyHostToDevice, s->stream));
  void* dst = nullptr;
  if (cudaMalloc(&dst, a.total * s->amp_bytes) != cudaSuccess) {
    cudaGetLastError();
    return set_error(s, QSV_ERR_OOM, "func_apply: allocation failed");
  }
  const unsigned grid = grid_for(s, a.total);
  if (is_c64(s))
    k_func<float><<<grid, QSV_THREADS, 0, s->stream>>>((const float2*)s->d_amp, (float2*)dst,
                                                       (const long long*)s->d_scratch, a);
  else
    k_func<double><<<grid, QSV_THREADS, 0, s->stream>>>((const double2*)s->d_amp, (double2*)dst,
                                                        (const long long*)s->d_scratch, a);
  rc = check_launch(s, "func_apply");
  if (rc) {
    cudaFree(dst);
    return rc;
  }
  QSV_CUDA(s, cudaStreamSynchronize(s->stream));
  cudaFree(s->d_amp);
  s->d_amp = dst;
  return QSV_OK;
}

int qsv_inner_product(qsv_state* a, qsv_state* b, double* re, double* im) {
  QSV_CHECK_HANDLE(a);
  QSV_CHECK_HANDLE(b);
  if (!re || !im) return set_error(a, QSV_ERR_INVALID, "null output");
  if (a->n != b->n) return set_error(a, QSV_ERR_INVALID, "states of %d and %d qubits", a->n, b->n);
  QSV_CUDA(a, cudaStreamSynchronize(b->stream));
  const uint64_t total = 1ull << a->n;
  const unsigned grid = grid_for(a, total, QSV_THREADS, 8);
  int rc = ensure_scratch(a, (size_t)grid * 2 * sizeof(double) + 2 * sizeof(double));
  if (rc) return rc;
  double* partial = (double*)a->d_scratch;
  double* col = partial + 2 * (size_t)grid;
  const bool a64 = is_c64(a), b64 = is_c64(b);
  if (a64 && b64)
    k_inner_partial<float, float><<<grid, QSV_THREADS, 0, a->stream>>>((const float2*)a->d_amp, (const float2*)b->d_amp, total, partial);
  else if (a64)
    k_inner_partial<float, double><<<grid, QSV_THREADS, 0, a->stream>>>((const float2*)a->d_amp, (const double2*)b->d_amp, total, partial);
  else if (b64)
    k_inner_partial<double, float><<<grid, QSV_THREADS, 0, a->stream>>>((const double2*)a->d_amp, (const float2*)b->d_amp, total, partial);
  else
    k_inner_partial<double, double><<<grid, QSV_THREADS, 0, a->stream>>>((const double2*)a->d_amp, (const double2*)b->d_amp, total, partial);
  rc = check_launch(a, "inner_partial");
  if (rc) return rc;
  k_columns_finish<<<1, 64, 0, a->stream>>>(partial, grid, 2, col);
  rc = check_launch(a, "inner_finish");
  if (rc) return rc;
  double h[2];
  QSV_CUDA(a, cudaMemcpyAsync(h, col, sizeof(h), cudaMemcpyDeviceToHost, a->stream));
  QSV_CUDA(a, cudaStreamSynchronize(a->stream));
  *re = h[0];
  *im = h[1];
  return QSV_OK;
}

}  // extern "C"

// ======================================================================================
// Allocation-free marginal probabilities
// ======================================================================================
// Some callers cannot allocate device memory at the moment they need probabilities: a
// host whose HBM is owned by another allocator (e.g. a framework's caching allocator
// that has reserved the whole device), or a latency-critical loop where an allocation
// (and the synchronisation it implies) is not allowed.  qsv_probabilities_static serves
// them: the caller passes the state and the output buffer, and the per-block partial
// sums go to the file-scope array below instead of a cudaMalloc'ed scratch.  Every GPU
// that loads this library holds the array (512 KiB) until the process exits.
constexpr size_t QSV_STATIC_PARTIALS = size_t(1) << 16;  // doubles: 512 KiB
static __device__ __align__(256) double g_static_partials[QSV_STATIC_PARTIALS];

namespace {
constexpr int QSV_MAX_DEVICES = 64;
std::mutex g_static_mu;
double* g_static_ptr[QSV_MAX_DEVICES] = {nullptr};
int g_static_sms[QSV_MAX_DEVICES] = {0};

// Device address of g_static_partials on the current device (looked up once per device;
// in host code the symbol's name is only a host-side stand-in).
int static_partials(double** out, int* sms) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error(nullptr, QSV_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= QSV_MAX_DEVICES) return set_error(nullptr, QSV_ERR_UNSUPPORTED, "device ordinal %d", dev);
  std::lock_guard<std::mutex> lk(g_static_mu);
  if (!g_static_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_partials);
    if (e != cudaSuccess)
      return set_error(nullptr, QSV_ERR_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    int count = 0;
    e = cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return set_error(nullptr, QSV_ERR_CUDA, "device attribute: %s", cudaGetErrorString(e));
    g_static_ptr[dev] = static_cast<double*>(p);
    g_static_sms[dev] = count;
  }
  *out = g_static_ptr[dev];
  *sms = g_static_sms[dev];
  return QSV_OK;
}

// The state and the output must be device memory of the current device, whose copy of
// the static array the kernels use: a buffer on another GPU (or in host memory) is
// rejected here rather than read over a peer link or faulted on.  Allocates nothing.
int check_current_device_buffer(const void* p, const char* what) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error(nullptr, QSV_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  cudaPointerAttributes at{};
  e = cudaPointerGetAttributes(&at, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(nullptr, QSV_ERR_INVALID, "%s: not a CUDA pointer (%s)", what, cudaGetErrorString(e));
  }
  if ((at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged) || at.device != dev)
    return set_error(nullptr, QSV_ERR_INVALID, "%s is not device memory of the current device (%d)", what, dev);
  return QSV_OK;
}

template <typename R>
int launch_probs_static(const void* d_amp, int n, int m, const int* pos_in_order, double* d_out,
                        cudaStream_t stream, double* partial, int sms) {
  ProbArgs a;
  a.m = m;
  a.npos = m;
  const uint64_t nbins = 1ull << m;
  a.nbins = nbins;
  a.nrest = 1ull << (n - m);
  for (int j = 0; j < m; ++j) {
    a.binbit[j] = 1ull << pos_in_order[j];
    a.pos[j] = pos_in_order[j];
  }
  std::sort(a.pos, a.pos + m);
  // Chunk the rest index so that nbins * nchunks partials fit the static array.
  const uint64_t target = std::min<uint64_t>((uint64_t)std::max(1, sms) * 32, QSV_STATIC_PARTIALS);
  uint64_t chunk = 4096;
  while (chunk < a.nrest && (nbins * ((a.nrest + chunk - 1) / chunk) > target)) chunk <<= 1;
  if (chunk > a.nrest) chunk = a.nrest;
  a.chunk = chunk;
  a.nchunks = (a.nrest + chunk - 1) / chunk;
  const uint64_t nblk = nbins * a.nchunks;
  if (nblk > QSV_STATIC_PARTIALS)
    return set_error(nullptr, QSV_ERR_INVALID, "%llu partial sums exceed the static scratch of %zu",
                     (unsigned long long)nblk, QSV_STATIC_PARTIALS);
  dim3 grid;
  grid.x = (unsigned)std::min<uint64_t>(nblk, 65535ull * 1024);
  grid.y = (unsigned)((nblk + grid.x - 1) / grid.x);
  k_probs_partial<R><<<grid, QSV_THREADS, 0, stream>>>((const CT<R>*)d_amp, a, partial);
  int rc = check_launch(nullptr, "probs_partial (static scratch)");
  if (rc) return rc;
  const unsigned fblocks = (unsigned)((nbins * 32 + QSV_THREADS - 1) / QSV_THREADS);
  k_probs_finish<<<fblocks, QSV_THREADS, 0, stream>>>(partial, a.nchunks, nbins, d_out);
  return check_launch(nullptr, "probs_finish (static scratch)");
}
}  // namespace

extern "C" int qsv_probabilities_static(const void* d_amp, int n, int dtype, int m, const int* qubits,
                                        double* d_out, void* stream) {
  if (!d_amp || !d_out) return set_error(nullptr, QSV_ERR_INVALID, "null state or output pointer");
  if (n < 1 || n > QSV_MAXN) return set_error(nullptr, QSV_ERR_INVALID, "n=%d outside [1, %d]", n, QSV_MAXN);
  if (dtype != QSV_C64 && dtype != QSV_C128) return set_error(nullptr, QSV_ERR_INVALID, "unknown dtype %d", dtype);
  if (m < 0 || m > n || m > QSV_STATIC_MAX_MEASURED)
    return set_error(nullptr, QSV_ERR_INVALID,
                     "%d measured qubits: the allocation-free path takes at most %d (2^%d outcomes)", m,
                     QSV_STATIC_MAX_MEASURED, QSV_STATIC_MAX_MEASURED);
  if (m > 0 && !qubits) return set_error(nullptr, QSV_ERR_INVALID, "null qubit list");
  int pos[QSV_MAXQ];
  uint64_t seen = 0;
  for (int j = 0; j < m; ++j) {
    const int q = qubits[j];
    if (q < 0 || q >= n) return set_error(nullptr, QSV_ERR_INVALID, "qubit index %d out of range for n=%d", q, n);
    const int p = n - 1 - q;
    if (seen & (1ull << p)) return set_error(nullptr, QSV_ERR_INVALID, "qubit %d repeated", q);
    seen |= 1ull << p;
    pos[j] = p;
  }
  int rc = check_current_device_buffer(d_amp, "the state");
  if (rc) return rc;
  rc = check_current_device_buffer(d_out, "the output");
  if (rc) return rc;
  double* partial = nullptr;
  int sms = 0;
  rc = static_partials(&partial, &sms);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  return dtype == QSV_C64 ? launch_probs_static<float>(d_amp, n, m, pos, d_out, st, partial, sms)
                          : launch_probs_static<double>(d_amp, n, m, pos, d_out, st, partial, sms);
}
