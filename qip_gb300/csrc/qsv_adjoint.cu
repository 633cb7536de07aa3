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

// Sum over the warp in the state's own precision (complex64 states: FP32, whose partial
// sums already carry FP32 rounding; FP64 shuffles and adds run at a fraction of the FP32
// rate here), returned as double for the FP64 accumulation that follows.
__device__ __forceinline__ double warp_sum_r(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return (double)v;
}
__device__ __forceinline__ double warp_sum_r(double v);

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double warp_sum_r(double v) { return warp_sum_d(v); }

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
    if (!QSV_IN_BOUNDS(i0 + hi, 1ull << a.n)) continue;
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
    if (!QSV_IN_BOUNDS(i0 + hi, 1ull << a.n)) continue;
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

// ---- segmented execution -----------------------------------------------------------
// A segment is a run of gates whose qubits lie in a set of LB bit positions (the
// segment's local bits, ascending in lpos, always containing the lowest address bits so
// a warp's accesses stay coalesced).  Each CTA takes chunks of one parameter set: a
// chunk is the 2^LB amplitudes with fixed values of the other n-LB bits, gathered into
// shared memory, and every gate of the segment is applied there before the chunk is
// scattered back: one pass over the state per segment instead of one per gate.
//
// Inside a segment the gates come in groups whose local bits number at most 3: a
// thread loads an item of 2^nb amplitudes (one value of the chunk's other bits), applies
// all the group's gates to it in registers, and stores it back — one shared-memory pass
// per group rather than per gate.
struct SegGate {
  int32_t tbit;   // target: index (0..nb-1) among its group's bits
  int32_t cbit;   // control: index among the group's bits, -1 if none
  int32_t g;      // gate index: matrices at mats[(g * nsets + s) * 4 ...]
  int32_t gp;     // (generator << 24) | parameter index; generator 0 none, 1 Y, 2 Z
};
struct SegGroup {
  int32_t nb;     // local bits of the group (1..3)
  int32_t bits;   // the bits (local positions), ascending, 8 bits each
  int32_t first;  // first gate of the group in the segment's gate table
  int32_t count;  // gates in the group (<= SEG_GROUP_GATES)
};
constexpr int SEG_THREADS = 512;
constexpr int SEG_MAX_GATES = 512;
constexpr int SEG_MAX_PARAMS = 256;
constexpr int SEG_GROUP_GATES = 8;

struct SegArgs {
  int n, nsets, lb, ngates, ngroups;
  int lpos[16];
  uint64_t nchunks;
};

// Shared-memory position of chunk element e: one padding amplitude every 16, so items
// whose group owns the lowest bits (lanes 8 or more amplitudes apart) spread over the
// banks instead of hitting two of them.
__device__ __forceinline__ int phys(int e) { return e + (e >> 4); }

// 2x2 matrix m on register bit J of an item (pairs with control bit c set, c >= 0).
template <typename R, int NB, int J>
__device__ __forceinline__ void reg_apply(CT<R>* a, int c, const CT<R> m[4]) {
#pragma unroll
  for (int i0 = 0; i0 < (1 << NB); ++i0) {
    if ((i0 >> J) & 1) continue;
    if (c >= 0 && !((i0 >> c) & 1)) continue;
    const int i1 = i0 | (1 << J);
    const CT<R> x = a[i0], y = a[i1];
    CT<R> o0, o1;
    o0.x = R(0); o0.y = R(0); o1 = o0;
    o0 = qsv_cfma(m[0], x, o0);
    o0 = qsv_cfma(m[1], y, o0);
    o1 = qsv_cfma(m[2], x, o1);
    o1 = qsv_cfma(m[3], y, o1);
    a[i0] = o0;
    a[i1] = o1;
  }
}

template <typename R, int NB>
__device__ __forceinline__ void reg_gate(CT<R>* a, int j, int c, const CT<R> m[4]) {
  if (j == 0) reg_apply<R, NB, 0>(a, c, m);
  if constexpr (NB > 1) if (j == 1) reg_apply<R, NB, 1>(a, c, m);
  if constexpr (NB > 2) if (j == 2) reg_apply<R, NB, 2>(a, c, m);
}

// Im <lambda| P |psi> over the pairs of register bit J (P = Z: gen 2, Y: gen 1).
template <typename R, int NB, int J>
__device__ __forceinline__ R reg_gen(const CT<R>* x, const CT<R>* l, int gen) {
  R part = R(0);
#pragma unroll
  for (int i0 = 0; i0 < (1 << NB); ++i0) {
    if ((i0 >> J) & 1) continue;
    const int i1 = i0 | (1 << J);
    const CT<R> x0 = x[i0], y0 = x[i1], l0 = l[i0], l1 = l[i1];
    if (gen == 2)
      part += (l0.x * x0.y - l0.y * x0.x) - (l1.x * y0.y - l1.y * y0.x);
    else
      part += (l1.x * x0.x + l1.y * x0.y) - (l0.x * y0.x + l0.y * y0.y);
  }
  return part;
}

template <typename R, int NB>
__device__ __forceinline__ R reg_gen_any(const CT<R>* x, const CT<R>* l, int j, int gen) {
  if (j == 0) return reg_gen<R, NB, 0>(x, l, gen);
  if constexpr (NB > 1) if (j == 1) return reg_gen<R, NB, 1>(x, l, gen);
  if constexpr (NB > 2) if (j == 2) return reg_gen<R, NB, 2>(x, l, gen);
  return R(0);
}

// Shared-memory offsets of an item's 2^NB amplitudes: item it -> zeros inserted at the
// group's bits; amplitude i adds the bits of i.
template <int NB>
__device__ __forceinline__ int item_base(int it, const int* gb) {
  int x = it;
#pragma unroll
  for (int j = 0; j < NB; ++j) x = ((x >> gb[j]) << (gb[j] + 1)) | (x & ((1 << gb[j]) - 1));
  return x;
}

template <typename R, int NB>
__device__ __forceinline__ void group_forward(CT<R>* v, int chunk, const int* gb, const SegGate* gsh,
                                              const CT<R>* msh, int first, int count) {
  constexpr int D = 1 << NB;
  int mb[NB];
#pragma unroll
  for (int j = 0; j < NB; ++j) mb[j] = 1 << gb[j];
  auto off = [&](int i) {
    int o = 0;
#pragma unroll
    for (int j = 0; j < NB; ++j)
      if ((i >> j) & 1) o |= mb[j];
    return o;
  };
  for (int it = threadIdx.x; it < (chunk >> NB); it += blockDim.x) {
    const int b = item_base<NB>(it, gb);
    CT<R> a[D];
#pragma unroll
    for (int i = 0; i < D; ++i) a[i] = v[phys(b + off(i))];
    for (int k = first; k < first + count; ++k) {
      const SegGate g = gsh[k];
      const CT<R> m[4] = {msh[4 * k], msh[4 * k + 1], msh[4 * k + 2], msh[4 * k + 3]};
      reg_gate<R, NB>(a, g.tbit, g.cbit, m);
    }
#pragma unroll
    for (int i = 0; i < D; ++i) v[phys(b + off(i))] = a[i];
  }
}

// Reverse over a group's gates on each item of psi and lambda; part[k - first] collects
// this thread's generator terms.
template <typename R, int NB>
__device__ __forceinline__ void group_adjoint(CT<R>* v, CT<R>* l, int chunk, const int* gb, const SegGate* gsh,
                                              const CT<R>* msh, int first, int count, R* part) {
  constexpr int D = 1 << NB;
  int mb[NB];
#pragma unroll
  for (int j = 0; j < NB; ++j) mb[j] = 1 << gb[j];
  auto off = [&](int i) {
    int o = 0;
#pragma unroll
    for (int j = 0; j < NB; ++j)
      if ((i >> j) & 1) o |= mb[j];
    return o;
  };
  for (int it = threadIdx.x; it < (chunk >> NB); it += blockDim.x) {
    const int b = item_base<NB>(it, gb);
    CT<R> a[D], la[D];
#pragma unroll
    for (int i = 0; i < D; ++i) {
      a[i] = v[phys(b + off(i))];
      la[i] = l[phys(b + off(i))];
    }
#pragma unroll
    for (int q = SEG_GROUP_GATES - 1; q >= 0; --q) {
      if (q >= count) continue;
      const int k = first + q;
      const SegGate g = gsh[k];
      const int gen = (g.gp >> 24) & 3;
      if (gen) part[q] += reg_gen_any<R, NB>(a, la, g.tbit, gen);
      const CT<R> m[4] = {msh[4 * k], msh[4 * k + 1], msh[4 * k + 2], msh[4 * k + 3]};
      reg_gate<R, NB>(a, g.tbit, g.cbit, m);
      reg_gate<R, NB>(la, g.tbit, g.cbit, m);
    }
#pragma unroll
    for (int i = 0; i < D; ++i) {
      v[phys(b + off(i))] = a[i];
      l[phys(b + off(i))] = la[i];
    }
  }
}

// Gathers a chunk (and optionally a second state's) into shared memory with GB loads per
// thread issued before the first shared store (the gather is latency-bound otherwise).
template <typename R, bool TWO>
__device__ __forceinline__ void seg_gather(const CT<R>* src, const CT<R>* src2, CT<R>* v, CT<R>* v2, int chunk,
                                           uint64_t base, const uint64_t* dlo, const uint64_t* dhi,
                                           [[maybe_unused]] uint64_t limit) {
  constexpr int GB = TWO ? (sizeof(R) == 4 ? 8 : 4) : (sizeof(R) == 4 ? 16 : 8);
  for (int e0 = threadIdx.x; e0 < chunk; e0 += GB * blockDim.x) {
    CT<R> t[GB], t2[TWO ? GB : 1];
#pragma unroll
    for (int j = 0; j < GB; ++j) {
      const int e = e0 + j * blockDim.x;
      if (e < chunk) {
        const uint64_t ad = base + dlo[e & 127] + dhi[e >> 7];
        if (!QSV_IN_BOUNDS(ad, limit)) continue;
        t[j] = src[ad];
        if constexpr (TWO) t2[j] = src2[ad];
      }
    }
#pragma unroll
    for (int j = 0; j < GB; ++j) {
      const int e = e0 + j * blockDim.x;
      if (e < chunk) {
        v[phys(e)] = t[j];
        if constexpr (TWO) v2[phys(e)] = t2[j];
      }
    }
  }
}

// The segment's gate records, groups and this set's matrices, staged in shared memory
// once per CTA (otherwise every gate starts with two dependent global loads).
template <typename R>
__device__ __forceinline__ void seg_stage(const SegGate* gates, const SegGroup* groups, const CT<R>* mats,
                                          const SegArgs& a, int s, SegGate* gsh, SegGroup* grsh, CT<R>* msh) {
  for (int k = threadIdx.x; k < a.ngates; k += blockDim.x) {
    const SegGate g = gates[k];
    gsh[k] = g;
    const CT<R>* mp = mats + ((uint64_t)g.g * a.nsets + s) * 4;
#pragma unroll
    for (int i = 0; i < 4; ++i) msh[4 * k + i] = mp[i];
  }
  for (int k = threadIdx.x; k < a.ngroups; k += blockDim.x) grsh[k] = groups[k];
}

template <typename R>
__device__ __forceinline__ void seg_tables(const SegArgs& a, uint64_t* dlo, uint64_t* dhi) {
  for (int i = threadIdx.x; i < 128; i += blockDim.x) {
    uint64_t lo = 0, hi = 0;
    for (int b = 0; b < 7; ++b)
      if ((i >> b) & 1) {
        if (b < a.lb) lo |= 1ull << a.lpos[b];
        if (7 + b < a.lb) hi |= 1ull << a.lpos[7 + b];
      }
    dlo[i] = lo;
    dhi[i] = hi;
  }
}

__device__ __forceinline__ void group_bits(const SegGroup& G, int* gb) {
  gb[0] = G.bits & 0xFF;
  gb[1] = (G.bits >> 8) & 0xFF;
  gb[2] = (G.bits >> 16) & 0xFF;
}

template <typename R>
__global__ void __launch_bounds__(SEG_THREADS, 2)
    k_seg_forward(CT<R>* __restrict__ psi, const CT<R>* __restrict__ mats, const SegGate* __restrict__ gates,
                  const SegGroup* __restrict__ groups, const __grid_constant__ SegArgs a) {
  extern __shared__ __align__(16) uint8_t seg_smem[];
  const int chunk = 1 << a.lb;
  CT<R>* v = reinterpret_cast<CT<R>*>(seg_smem);
  CT<R>* msh = v + phys(chunk);                             // [ngates][4] this set's matrices
  SegGate* gsh = reinterpret_cast<SegGate*>(msh + 4 * a.ngates);
  SegGroup* grsh = reinterpret_cast<SegGroup*>(gsh + a.ngates);
  __shared__ uint64_t dlo[128], dhi[128];
  const int s = blockIdx.y;
  CT<R>* st = psi + ((uint64_t)s << a.n);
  seg_tables<R>(a, dlo, dhi);
  seg_stage<R>(gates, groups, mats, a, s, gsh, grsh, msh);
  __syncthreads();
  for (uint64_t ch = blockIdx.x; ch < a.nchunks; ch += gridDim.x) {
    const uint64_t base = qsv_insert_zeros(ch, a.lpos, a.lb);
    seg_gather<R, false>(st, nullptr, v, nullptr, chunk, base, dlo, dhi, 1ull << a.n);
    __syncthreads();
    for (int q = 0; q < a.ngroups; ++q) {
      const SegGroup G = grsh[q];
      int gb[3];
      group_bits(G, gb);
      if (G.nb == 1)
        group_forward<R, 1>(v, chunk, gb, gsh, msh, G.first, G.count);
      else if (G.nb == 2)
        group_forward<R, 2>(v, chunk, gb, gsh, msh, G.first, G.count);
      else
        group_forward<R, 3>(v, chunk, gb, gsh, msh, G.first, G.count);
      __syncthreads();
    }
    for (int e = threadIdx.x; e < chunk; e += blockDim.x)
      if (QSV_IN_BOUNDS(base + dlo[e & 127] + dhi[e >> 7], 1ull << a.n)) st[base + dlo[e & 127] + dhi[e >> 7]] = v[phys(e)];
    __syncthreads();
  }
}

// Reverse sweep over one segment: groups last to first, each group's gates last to
// first: [generator: Im<lambda| P |psi>]; psi, lambda <- M psi, M lambda (M = U^+).  Per
// warp FP64 accumulators in shared memory, one atomicAdd per parameter per CTA.
// Two CTAs per SM for complex64 (registers capped at 64); complex128 items need more.
template <typename R>
__global__ void __launch_bounds__(SEG_THREADS, sizeof(R) == 4 ? 2 : 1)
    k_seg_adjoint(CT<R>* __restrict__ psi, CT<R>* __restrict__ lam, const CT<R>* __restrict__ mats_dagger,
                  const SegGate* __restrict__ gates, const SegGroup* __restrict__ groups,
                  const __grid_constant__ SegArgs a, double* __restrict__ grads, int grad_stride) {
  extern __shared__ __align__(16) uint8_t seg_smem[];
  const int chunk = 1 << a.lb;
  CT<R>* v = reinterpret_cast<CT<R>*>(seg_smem);
  CT<R>* l = v + phys(chunk);
  const int nrows = min(a.ngates, SEG_MAX_PARAMS);  // generator slots (<= gates)
  double* accw = reinterpret_cast<double*>(l + phys(chunk));  // [nrows][16 warps]
  CT<R>* msh = reinterpret_cast<CT<R>*>(accw + nrows * 16);  // [ngates][4]
  SegGate* gsh = reinterpret_cast<SegGate*>(msh + 4 * a.ngates);
  SegGroup* grsh = reinterpret_cast<SegGroup*>(gsh + a.ngates);
  __shared__ uint64_t dlo[128], dhi[128];
  __shared__ int slot_of[SEG_MAX_GATES];
  const int s = blockIdx.y;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nwarps = blockDim.x >> 5;
  CT<R>* sp = psi + ((uint64_t)s << a.n);
  CT<R>* sl = lam + ((uint64_t)s << a.n);
  seg_tables<R>(a, dlo, dhi);
  seg_stage<R>(gates, groups, mats_dagger, a, s, gsh, grsh, msh);
  if (threadIdx.x == 0) {
    int np = 0;
    for (int k = 0; k < a.ngates; ++k) slot_of[k] = (((gates[k].gp >> 24) & 3) && np < nrows) ? np++ : -1;
  }
  for (int i = threadIdx.x; i < nrows * 16; i += blockDim.x) accw[i] = 0.0;
  __syncthreads();
  for (uint64_t ch = blockIdx.x; ch < a.nchunks; ch += gridDim.x) {
    const uint64_t base = qsv_insert_zeros(ch, a.lpos, a.lb);
    seg_gather<R, true>(sp, sl, v, l, chunk, base, dlo, dhi, 1ull << a.n);
    __syncthreads();
    for (int q = a.ngroups - 1; q >= 0; --q) {
      const SegGroup G = grsh[q];
      int gb[3];
      group_bits(G, gb);
      R part[SEG_GROUP_GATES];
#pragma unroll
      for (int i = 0; i < SEG_GROUP_GATES; ++i) part[i] = R(0);
      if (G.nb == 1)
        group_adjoint<R, 1>(v, l, chunk, gb, gsh, msh, G.first, G.count, part);
      else if (G.nb == 2)
        group_adjoint<R, 2>(v, l, chunk, gb, gsh, msh, G.first, G.count, part);
      else
        group_adjoint<R, 3>(v, l, chunk, gb, gsh, msh, G.first, G.count, part);
#pragma unroll
      for (int i = 0; i < SEG_GROUP_GATES; ++i) {
        if (i >= G.count) continue;
        const int k = G.first + i;
        if (!((gsh[k].gp >> 24) & 3)) continue;
        const double w = warp_sum_r(part[i]);
        if (lane == 0 && slot_of[k] >= 0) accw[slot_of[k] * 16 + warp] += w;
      }
      __syncthreads();
    }
    for (int e = threadIdx.x; e < chunk; e += blockDim.x) {
      const uint64_t ad = base + dlo[e & 127] + dhi[e >> 7];
      if (!QSV_IN_BOUNDS(ad, 1ull << a.n)) continue;
      sp[ad] = v[phys(e)];
      sl[ad] = l[phys(e)];
    }
    __syncthreads();
  }
  for (int k = threadIdx.x; k < a.ngates; k += blockDim.x) {
    const int slot = slot_of[k];
    if (slot < 0) continue;
    double sum = 0.0;
    for (int w = 0; w < nwarps; ++w) sum += accw[slot * 16 + w];
    atomicAdd(&grads[(uint64_t)s * grad_stride + (gates[k].gp & 0xFFFFFF)], sum);
  }
}

}  // namespace

namespace qsv {
int oob_take_adjoint(unsigned long long* count, unsigned long long* first) {
#ifdef QSV_BOUNDS_CHECK
  return qsv_oob_take_unit(count, first);
#else
  (void)count;
  (void)first;
  return 0;
#endif
}
}  // namespace qsv

namespace {

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

// Per-gate, per-set 2x2 matrices of rotation circuits: gate g of kind 0 (RY(theta)),
// 1 (RZ(theta)) or 2 (CNOT: X on the target) with angle thetas[s * nparams + param[g]];
// U[(g * nsets + s) * 4 + ...] row-major and Ud = U^+, in the batch's precision.
template <typename R>
__global__ void k_batch_rotations(const double* __restrict__ thetas, int nsets, int nparams, int ngates,
                                  const int2* __restrict__ kind_param, CT<R>* __restrict__ U,
                                  CT<R>* __restrict__ Ud) {
  const uint64_t total = (uint64_t)ngates * nsets;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const int g = (int)(i / nsets), s = (int)(i % nsets);
    const int2 kp = kind_param[g];
    double m[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // re/im of u00, u01, u10, u11
    if (kp.x == 2) {
      m[2] = 1.0;
      m[4] = 1.0;
    } else {
      double sn, cs;
      sincos(0.5 * thetas[(size_t)s * nparams + kp.y], &sn, &cs);
      if (kp.x == 0) {
        m[0] = cs;
        m[2] = -sn;
        m[4] = sn;
        m[6] = cs;
      } else {
        m[0] = cs;
        m[1] = -sn;
        m[6] = cs;
        m[7] = sn;
      }
    }
    CT<R>* u = U + i * 4;
    CT<R>* ud = Ud + i * 4;
    for (int e = 0; e < 4; ++e) u[e] = {(R)m[2 * e], (R)m[2 * e + 1]};
    // (U^+)[r][c] = conj(U[c][r])
    ud[0] = {(R)m[0], (R)-m[1]};
    ud[1] = {(R)m[4], (R)-m[5]};
    ud[2] = {(R)m[2], (R)-m[3]};
    ud[3] = {(R)m[6], (R)-m[7]};
  }
}

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

int qsv_batch_rotation_matrices(const double* thetas, int nsets, int nparams, int ngates, const int* kind_param,
                                int dtype, void* U, void* Ud, void* stream) {
  if (!thetas || !kind_param || !U || !Ud || nsets < 1 || ngates < 0 || nparams < 0)
    return set_error(nullptr, QSV_ERR_INVALID, "bad rotation-matrix arguments");
  if (ngates == 0) return QSV_OK;
  const uint64_t total = (uint64_t)ngates * nsets;
  const unsigned grid = (unsigned)std::min<uint64_t>((total + QSV_THREADS - 1) / QSV_THREADS, (uint64_t)sms() * 8);
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == QSV_C64)
    k_batch_rotations<float><<<grid, QSV_THREADS, 0, st>>>(thetas, nsets, nparams, ngates, (const int2*)kind_param,
                                                           (float2*)U, (float2*)Ud);
  else if (dtype == QSV_C128)
    k_batch_rotations<double><<<grid, QSV_THREADS, 0, st>>>(thetas, nsets, nparams, ngates, (const int2*)kind_param,
                                                            (double2*)U, (double2*)Ud);
  else
    return set_error(nullptr, QSV_ERR_INVALID, "unknown dtype %d", dtype);
  return launch_check("batch_rotations");
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

// ---- segmented execution ------------------------------------------------------------
namespace {
int seg_args(int n, int nsets, int dtype, int lb, const int* lpos, int ngroups, int ngates, bool two, SegArgs& a,
             size_t& smem) {
  if (n < 1 || n > QSV_MAXN || nsets < 1 || nsets > 65535 || !lpos || ngates < 0 || ngates > SEG_MAX_GATES ||
      ngroups < 0 || ngroups > ngates)
    return set_error(nullptr, QSV_ERR_INVALID, "bad segment (n=%d nsets=%d groups=%d gates=%d)", n, nsets, ngroups,
                     ngates);
  if (dtype != QSV_C64 && dtype != QSV_C128) return set_error(nullptr, QSV_ERR_INVALID, "unknown dtype %d", dtype);
  const size_t amp = dtype == QSV_C64 ? 8 : 16;
  const int lbmax = dtype == QSV_C64 ? 13 : 12;
  if (lb < 1 || lb > n || lb > lbmax) return set_error(nullptr, QSV_ERR_INVALID, "local bits %d outside [1, %d]", lb, lbmax);
  for (int i = 0; i < lb; ++i) {
    if (lpos[i] < 0 || lpos[i] >= n || (i > 0 && lpos[i] <= lpos[i - 1]))
      return set_error(nullptr, QSV_ERR_INVALID, "local bit positions must ascend within [0, n)");
    a.lpos[i] = lpos[i];
  }
  a.n = n;
  a.nsets = nsets;
  a.lb = lb;
  a.ngates = ngates;
  a.ngroups = ngroups;
  a.nchunks = 1ull << (n - lb);
  const size_t padded = ((size_t)1 << lb) + ((size_t)1 << lb) / 16;  // one padding amplitude per 16
  smem = padded * amp * (two ? 2 : 1) +
         (two ? (size_t)std::min(ngates, SEG_MAX_PARAMS) * 16 * sizeof(double) : 0) +
         (size_t)ngates * (4 * amp + sizeof(SegGate) + sizeof(SegGroup));
  return QSV_OK;
}

template <typename K>
int seg_config(K kernel, size_t smem, const char* what) {
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return set_error(nullptr, QSV_ERR_CUDA, "%s smem attribute: %s", what, cudaGetErrorString(e));
  return QSV_OK;
}

dim3 seg_grid(uint64_t nchunks, int nsets, int per_sm) {
  uint64_t want = ((uint64_t)sms() * per_sm * 4 + nsets - 1) / nsets;
  if (want < 1) want = 1;
  return dim3((unsigned)std::min<uint64_t>(want, nchunks), (unsigned)nsets);
}
}  // namespace

extern "C" {

int qsv_batch_segment_forward(void* psi, int nsets, int n, int dtype, int lb, const int* lpos, int ngroups,
                              const void* groups_dev, int ngates, const void* gates_dev, const void* mats,
                              void* stream) {
  if (!psi || !mats || (ngates > 0 && (!gates_dev || !groups_dev)))
    return set_error(nullptr, QSV_ERR_INVALID, "null pointer");
  SegArgs a;
  size_t smem = 0;
  int rc = seg_args(n, nsets, dtype, lb, lpos, ngroups, ngates, false, a, smem);
  if (rc || ngates == 0) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const dim3 grid = seg_grid(a.nchunks, nsets, 2);
  if (dtype == QSV_C64) {
    if ((rc = seg_config(k_seg_forward<float>, smem, "segment_forward"))) return rc;
    k_seg_forward<float><<<grid, SEG_THREADS, smem, st>>>((float2*)psi, (const float2*)mats,
                                                          (const SegGate*)gates_dev, (const SegGroup*)groups_dev, a);
  } else {
    if ((rc = seg_config(k_seg_forward<double>, smem, "segment_forward"))) return rc;
    k_seg_forward<double><<<grid, SEG_THREADS, smem, st>>>((double2*)psi, (const double2*)mats,
                                                           (const SegGate*)gates_dev, (const SegGroup*)groups_dev, a);
  }
  return launch_check("segment_forward");
}

int qsv_batch_segment_adjoint(void* psi, void* lam, int nsets, int n, int dtype, int lb, const int* lpos, int ngroups,
                              const void* groups_dev, int ngates, const void* gates_dev, const void* mats_dagger,
                              double* grads, int grad_stride, void* stream) {
  if (!psi || !lam || !mats_dagger || !grads || (ngates > 0 && (!gates_dev || !groups_dev)))
    return set_error(nullptr, QSV_ERR_INVALID, "null pointer");
  SegArgs a;
  size_t smem = 0;
  int rc = seg_args(n, nsets, dtype, lb, lpos, ngroups, ngates, true, a, smem);
  if (rc || ngates == 0) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const dim3 grid = seg_grid(a.nchunks, nsets, 2);
  if (dtype == QSV_C64) {
    if ((rc = seg_config(k_seg_adjoint<float>, smem, "segment_adjoint"))) return rc;
    k_seg_adjoint<float><<<grid, SEG_THREADS, smem, st>>>((float2*)psi, (float2*)lam, (const float2*)mats_dagger,
                                                          (const SegGate*)gates_dev, (const SegGroup*)groups_dev, a,
                                                          grads, grad_stride);
  } else {
    if ((rc = seg_config(k_seg_adjoint<double>, smem, "segment_adjoint"))) return rc;
    k_seg_adjoint<double><<<grid, SEG_THREADS, smem, st>>>((double2*)psi, (double2*)lam,
                                                           (const double2*)mats_dagger, (const SegGate*)gates_dev,
                                                           (const SegGroup*)groups_dev, a, grads, grad_stride);
  }
  return launch_check("segment_adjoint");
}

}  // extern "C"
