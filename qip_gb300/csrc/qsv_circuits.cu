// Many independent small circuits in one persistent launch.
//
// One CTA per SM takes circuits from a global counter (an atomicAdd work queue: no
// CTA ever waits on another).  The host orders circuits by estimated cost, longest
// first, so the tail of the launch is short.  A circuit of n <= 14 qubits lives entirely
// in shared memory (2^14 complex64 = 128 KiB): its product-state input is built there
// from the per-qubit feeds, every gate is applied there, and the final state is
// written to global memory once.
//
// Larger circuits (15 <= n <= 24) are streamed through the same shared buffer by
// segments.  The host cuts the gate list into maximal runs whose qubits, together with
// address bits 0..4, fit in 14 bit positions (the segment's local set, completed from
// the lowest remaining positions) and rewrites those gates' qubits as local indices.
// For each segment the CTA gathers every chunk of 2^14 amplitudes (fixed values of the
// other n-14 bits; lanes walk address bits 0..4, so accesses stay coalesced) into
// shared memory, applies the segment's gates there and scatters the chunk back: one
// pass over the state per segment instead of one per gate.  The first segment builds
// its chunks from the feeds instead of reading them.  Each circuit records device
// timestamps (%globaltimer) when its CTA starts and finishes it.
//
// Large circuits run on a whole thread-block cluster.  The kernel is launched in
// clusters of CS CTAs (CS = 6 by default; QSV_CIRCUIT_CLUSTER=1..8 overrides; the
// clusters are co-scheduled by the hardware).  First each cluster takes circuits of
// n >= 14 + log2(2 CS) (at least two chunks per CTA; the host puts them first, largest
// first) from one counter: rank 0
// draws the index, the others read it from rank 0's shared memory; every CTA of the
// cluster streams the chunks ch = rank, rank + CS, ... of each segment, and a cluster
// barrier (barrier.cluster, release/acquire, no software spin) separates segments.  A
// circuit's latency is then about 1/CS of one CTA's.  Then every CTA takes the remaining
// circuits (smaller streamed ones and the shared-memory ones) from a second counter, one
// CTA each, as before.
//
// The launch (counter reset + kernel) is captured once into a CUDA graph owned by the
// batch object and replayed by qsv_circuits_run.

#include <cooperative_groups.h>

#include <algorithm>
#include <cstdlib>
#include <new>
#include <vector>

#include "qsv_internal.cuh"

using namespace qsv;

namespace {

constexpr int CB_THREADS = 512;
constexpr int CB_SMEM_QUBITS = 14;
constexpr int CB_MAX_QUBITS = 24;

enum GateKind : int32_t { G_DENSE1 = 0, G_PHASE1 = 1, G_X = 2, G_CX = 3, G_CSWAP = 4 };

}  // namespace

// Record layouts qsv_gate_rec / qsv_circuit_rec are declared in include/qsv.h
// (mirrored by qip_gb300/batch.py).

namespace {
// One segment of a streamed circuit (see above): its gates and its local bit positions.
struct SegmentRec {
  int32_t gate_begin, gate_end;  // absolute indices into the gate array
  int32_t lpos[CB_SMEM_QUBITS];  // ascending; lpos[0..4] = 0..4
};
static_assert(sizeof(SegmentRec) == 64, "segment record layout");
}  // namespace

struct qsv_circuits {
  int ncirc = 0;
  SegmentRec* d_segs = nullptr;
  int2* d_segidx = nullptr;  // per circuit: [first, last) segment (streamed circuits only)
  qsv_gate_rec* d_gates = nullptr;
  qsv_circuit_rec* d_circs = nullptr;
  float2* d_feeds = nullptr;
  float2* d_states = nullptr;
  unsigned long long* d_times = nullptr;
  int* d_counter = nullptr;  // [0] clustered circuits, [1] the others
  int nbig = 0;              // leading circuits run by a whole cluster
  int cluster = 1;
  size_t state_amps = 0;
  std::vector<qsv_circuit_rec> h_circs;
  cudaGraphExec_t graph = nullptr;
  cudaStream_t graph_stream = nullptr;
  int sm_count = 0;
};

namespace {

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint64_t ins0(uint64_t g, int p) {
  return ((g >> p) << (p + 1)) | (g & ((1ull << p) - 1ull));
}

// Applies one gate to a state of 2^n amplitudes at v (shared or global memory).
__device__ __forceinline__ void apply_gate(float2* v, int n, const qsv_gate_rec& g) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int p0 = n - 1 - g.q0;
  switch (g.kind) {
    case G_DENSE1: {
      const float2 m00 = make_float2(g.m[0], g.m[1]), m01 = make_float2(g.m[2], g.m[3]);
      const float2 m10 = make_float2(g.m[4], g.m[5]), m11 = make_float2(g.m[6], g.m[7]);
      const uint64_t pairs = 1ull << (n - 1), hi = 1ull << p0;
      for (uint64_t k = tid; k < pairs; k += nt) {
        const uint64_t i0 = ins0(k, p0);
        const float2 x = v[i0], y = v[i0 + hi];
        float2 o0 = make_float2(0.f, 0.f), o1 = o0;
        o0 = qsv_cfma(m00, x, o0);
        o0 = qsv_cfma(m01, y, o0);
        o1 = qsv_cfma(m10, x, o1);
        o1 = qsv_cfma(m11, y, o1);
        v[i0] = o0;
        v[i0 + hi] = o1;
      }
      break;
    }
    case G_PHASE1: {
      const float2 ph = make_float2(g.m[0], g.m[1]);
      const uint64_t cnt = 1ull << (n - 1), hi = 1ull << p0;
      for (uint64_t k = tid; k < cnt; k += nt) {
        const uint64_t i = ins0(k, p0) | hi;
        v[i] = qsv_cmul(ph, v[i]);
      }
      break;
    }
    case G_X: {
      const uint64_t pairs = 1ull << (n - 1), hi = 1ull << p0;
      for (uint64_t k = tid; k < pairs; k += nt) {
        const uint64_t i0 = ins0(k, p0);
        const float2 x = v[i0];
        v[i0] = v[i0 + hi];
        v[i0 + hi] = x;
      }
      break;
    }
    case G_CX: {
      const int pc = n - 1 - g.q1;
      const int lo = min(p0, pc), hp = max(p0, pc);
      const uint64_t cnt = 1ull << (n - 2), tb = 1ull << p0, cb = 1ull << pc;
      for (uint64_t k = tid; k < cnt; k += nt) {
        const uint64_t i0 = ins0(ins0(k, lo), hp) | cb;
        const float2 x = v[i0];
        v[i0] = v[i0 + tb];
        v[i0 + tb] = x;
      }
      break;
    }
    case G_CSWAP: {
      const int pc = n - 1 - g.q0, pa = n - 1 - g.q1, pb = n - 1 - g.q2;
      int s0 = pc, s1 = pa, s2 = pb;  // sort ascending for zero insertion
      if (s0 > s1) { const int t = s0; s0 = s1; s1 = t; }
      if (s1 > s2) { const int t = s1; s1 = s2; s2 = t; }
      if (s0 > s1) { const int t = s0; s0 = s1; s1 = t; }
      const uint64_t cnt = 1ull << (n - 3);
      for (uint64_t k = tid; k < cnt; k += nt) {
        const uint64_t base = ins0(ins0(ins0(k, s0), s1), s2) | (1ull << pc);
        const uint64_t ia = base | (1ull << pa), ib = base | (1ull << pb);
        const float2 x = v[ia];
        v[ia] = v[ib];
        v[ib] = x;
      }
      break;
    }
    default:
      break;
  }
}

// Product state: amp[i] = prod_q feed_q[bit of qubit q in i].
__device__ __forceinline__ void build_product(float2* v, int n, const float2* feed) {
  const uint64_t total = 1ull << n;
  for (uint64_t i = threadIdx.x; i < total; i += blockDim.x) {
    float2 acc = make_float2(1.f, 0.f);
    for (int q = 0; q < n; ++q) acc = qsv_cmul(acc, feed[2 * q + ((i >> (n - 1 - q)) & 1ull)]);
    v[i] = acc;
  }
}

// Streams a circuit of n > 14 qubits through the shared buffer segment by segment.
// With clustered, the CTAs of the cluster share the chunks (this CTA: rank, rank + size,
// ...) and meet at a cluster barrier after each segment; else one CTA does all chunks.
__device__ void run_segments(float2* sv, float2* out, int n, const qsv_gate_rec* gates, const SegmentRec* segs,
                             int2 range, const float2* feed, bool clustered) {
  namespace cg = cooperative_groups;
  const uint64_t crank = clustered ? cg::this_cluster().block_rank() : 0;
  const uint64_t csize = clustered ? cg::this_cluster().num_blocks() : 1;
  __shared__ uint64_t dlo[128], dhi[128];  // address offset of chunk element bits 0..6 / 7..13
  constexpr int CHUNK = 1 << CB_SMEM_QUBITS;
  const uint64_t nchunks = 1ull << (n - CB_SMEM_QUBITS);
  for (int si = range.x; si < range.y; ++si) {
    const SegmentRec sg = segs[si];
    if (threadIdx.x < 128) {
      uint64_t lo = 0, hi = 0;
      for (int b = 0; b < 7; ++b)
        if ((threadIdx.x >> b) & 1) {
          lo |= 1ull << sg.lpos[b];
          hi |= 1ull << sg.lpos[7 + b];
        }
      dlo[threadIdx.x] = lo;
      dhi[threadIdx.x] = hi;
    }
    __syncthreads();
    for (uint64_t ch = crank; ch < nchunks; ch += csize) {
      const uint64_t base = qsv_insert_zeros(ch, sg.lpos, CB_SMEM_QUBITS);
      if (si == range.x) {
        for (int e = threadIdx.x; e < CHUNK; e += blockDim.x) {
          const uint64_t i = base + dlo[e & 127] + dhi[e >> 7];
          float2 acc = make_float2(1.f, 0.f);
          for (int q = 0; q < n; ++q) acc = qsv_cmul(acc, feed[2 * q + ((i >> (n - 1 - q)) & 1ull)]);
          sv[e] = acc;
        }
      } else {
        // All of a thread's loads issued before the first shared store (the gather is
        // latency-bound: one chunk in flight per SM).
        constexpr int PER = CHUNK / CB_THREADS;
        float2 t[PER];
#pragma unroll
        for (int j = 0; j < PER; ++j) {
          const int e = threadIdx.x + j * CB_THREADS;
          t[j] = QSV_IN_BOUNDS(base + dlo[e & 127] + dhi[e >> 7], 1ull << n) ? out[base + dlo[e & 127] + dhi[e >> 7]]
                                                                            : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int j = 0; j < PER; ++j) sv[threadIdx.x + j * CB_THREADS] = t[j];
      }
      __syncthreads();
      for (int k = sg.gate_begin; k < sg.gate_end; ++k) {
        const qsv_gate_rec g = gates[k];
        apply_gate(sv, CB_SMEM_QUBITS, g);
        __syncthreads();
      }
#pragma unroll 8
      for (int e = threadIdx.x; e < CHUNK; e += blockDim.x)
        if (QSV_IN_BOUNDS(base + dlo[e & 127] + dhi[e >> 7], 1ull << n)) out[base + dlo[e & 127] + dhi[e >> 7]] = sv[e];
      __syncthreads();
    }
    if (clustered) {
      // The next segment's chunks overlap this one's across CTAs.
      __threadfence();
      cg::this_cluster().sync();
    }
  }
}

__global__ void __launch_bounds__(CB_THREADS, 1)
    k_circuits(const qsv_gate_rec* __restrict__ gates, const qsv_circuit_rec* __restrict__ circs, int ncirc,
               int nbig, float2* __restrict__ states, const float2* __restrict__ feeds,
               unsigned long long* __restrict__ times, int* __restrict__ counter, const SegmentRec* __restrict__ segs,
               const int2* __restrict__ segidx) {
  namespace cg = cooperative_groups;
  extern __shared__ float2 sv[];
  __shared__ int cur;
  cg::cluster_group cluster = cg::this_cluster();
  const bool lead = cluster.block_rank() == 0;
  // Circuits [0, nbig): one cluster each (every CTA of the cluster sees the same index
  // and the same number of iterations, so the cluster barriers always match).
  for (;;) {
    if (lead && threadIdx.x == 0) cur = atomicAdd(&counter[0], 1);
    cluster.sync();
    const int c = *cluster.map_shared_rank(&cur, 0);
    cluster.sync();  // everyone has read the index before rank 0 draws the next
    if (c >= nbig) break;
    const qsv_circuit_rec cr = circs[c];
    if (lead && threadIdx.x == 0) times[2 * (size_t)c] = gtimer();
    run_segments(sv, states + cr.state_offset, cr.n, gates, segs, segidx[c], feeds + cr.feed_offset, true);
    if (lead && threadIdx.x == 0) times[2 * (size_t)c + 1] = gtimer();
  }
  // The rest, one CTA each.
  for (;;) {
    if (threadIdx.x == 0) cur = nbig + atomicAdd(&counter[1], 1);
    __syncthreads();
    const int c = cur;
    __syncthreads();
    if (c >= ncirc) break;
    const qsv_circuit_rec cr = circs[c];
    if (threadIdx.x == 0) times[2 * (size_t)c] = gtimer();
    const qsv_gate_rec* gl = gates + cr.gate_offset;
    float2* out = states + cr.state_offset;
    if (cr.n <= CB_SMEM_QUBITS) {
      build_product(sv, cr.n, feeds + cr.feed_offset);
      __syncthreads();
      for (int k = 0; k < cr.ngates; ++k) {
        const qsv_gate_rec g = gl[k];
        apply_gate(sv, cr.n, g);
        __syncthreads();
      }
      const uint64_t total = 1ull << cr.n;
      for (uint64_t i = threadIdx.x; i < total; i += blockDim.x) out[i] = sv[i];
    } else {
      run_segments(sv, out, cr.n, gates, segs, segidx[c], feeds + cr.feed_offset, false);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      times[2 * (size_t)c + 1] = gtimer();
    }
  }
}

int capture(qsv_circuits* b, cudaStream_t stream) {
  const size_t smem = sizeof(float2) << CB_SMEM_QUBITS;
  cudaError_t e = cudaFuncSetAttribute(k_circuits, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return set_error(nullptr, QSV_ERR_CUDA, "smem attribute: %s", cudaGetErrorString(e));
  cudaGraph_t g = nullptr;
  // Grid: as many clusters as fit at once (one CTA per SM), at most one CTA per circuit
  // (rounded up to whole clusters).
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr;
  attr.id = cudaLaunchAttributeClusterDimension;
  attr.val.clusterDim.x = (unsigned)b->cluster;
  attr.val.clusterDim.y = 1;
  attr.val.clusterDim.z = 1;
  cfg.blockDim = dim3(CB_THREADS);
  cfg.dynamicSmemBytes = smem;
  cfg.attrs = &attr;
  cfg.numAttrs = 1;
  cfg.gridDim = dim3((unsigned)b->cluster);
  int clusters = 0;
  e = cudaOccupancyMaxActiveClusters(&clusters, k_circuits, &cfg);
  if (e != cudaSuccess || clusters < 1) {
    cudaGetLastError();
    clusters = std::max(1, b->sm_count / b->cluster);
  }
  const int need = (b->ncirc + b->cluster - 1) / b->cluster;
  cfg.gridDim = dim3((unsigned)(std::min(clusters, need) * b->cluster));
  cfg.stream = stream;
  e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return set_error(nullptr, QSV_ERR_CUDA, "begin capture: %s", cudaGetErrorString(e));
  cudaMemsetAsync(b->d_counter, 0, 2 * sizeof(int), stream);
  cudaError_t le = cudaLaunchKernelEx(&cfg, k_circuits, (const qsv_gate_rec*)b->d_gates, (const qsv_circuit_rec*)b->d_circs,
                                      b->ncirc, b->nbig, b->d_states, (const float2*)b->d_feeds, b->d_times,
                                      b->d_counter, (const SegmentRec*)b->d_segs, (const int2*)b->d_segidx);
  if (le == cudaSuccess) le = cudaGetLastError();
  e = cudaStreamEndCapture(stream, &g);
  if (le != cudaSuccess || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return set_error(nullptr, QSV_ERR_CUDA, "capture: %s", cudaGetErrorString(le != cudaSuccess ? le : e));
  }
  e = cudaGraphInstantiate(&b->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return set_error(nullptr, QSV_ERR_CUDA, "instantiate: %s", cudaGetErrorString(e));
  b->graph_stream = stream;
  return QSV_OK;
}

}  // namespace

namespace qsv {
int oob_take_circuits(unsigned long long* count, unsigned long long* first) {
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

int qsv_circuits_create(const void* gates, int64_t ngates, const void* circuits, int ncirc, const void* feeds,
                        int64_t nfeeds, qsv_circuits** out) {
  if (!out || !gates || !circuits || !feeds || ncirc < 1 || ngates < 0 || nfeeds < 0)
    return set_error(nullptr, QSV_ERR_INVALID, "bad circuit batch");
  *out = nullptr;
  const auto* gr = static_cast<const qsv_gate_rec*>(gates);
  const auto* cr = static_cast<const qsv_circuit_rec*>(circuits);
  size_t amps = 0;
  for (int c = 0; c < ncirc; ++c) {
    const qsv_circuit_rec& r = cr[c];
    if (r.n < 3 || r.n > CB_MAX_QUBITS || r.ngates < 0 || r.gate_offset < 0 || r.gate_offset + r.ngates > ngates ||
        r.feed_offset < 0 || r.feed_offset + 2 * r.n > nfeeds || r.state_offset < 0)
      return set_error(nullptr, QSV_ERR_INVALID, "circuit %d: bad record (n=%d)", c, r.n);
    amps = std::max(amps, (size_t)r.state_offset + ((size_t)1 << r.n));
    for (int64_t k = r.gate_offset; k < r.gate_offset + r.ngates; ++k) {
      const qsv_gate_rec& g = gr[k];
      const int need = g.kind == G_CX ? 2 : (g.kind == G_CSWAP ? 3 : 1);
      const int qs[3] = {g.q0, g.q1, g.q2};
      if (g.kind < G_DENSE1 || g.kind > G_CSWAP)
        return set_error(nullptr, QSV_ERR_INVALID, "circuit %d gate %lld: kind %d", c, (long long)k, g.kind);
      for (int i = 0; i < need; ++i)
        if (qs[i] < 0 || qs[i] >= r.n)
          return set_error(nullptr, QSV_ERR_INVALID, "circuit %d gate %lld: qubit %d", c, (long long)k, qs[i]);
      for (int i = 0; i < need; ++i)
        for (int j = i + 1; j < need; ++j)
          if (qs[i] == qs[j])
            return set_error(nullptr, QSV_ERR_INVALID, "circuit %d gate %lld: repeated qubit", c, (long long)k);
    }
  }
  // Segments of the streamed circuits; their gates are rewritten to local indices.
  std::vector<qsv_gate_rec> gv(gr, gr + ngates);
  std::vector<SegmentRec> segs;
  std::vector<int2> segidx((size_t)ncirc, make_int2(0, 0));
  for (int c = 0; c < ncirc; ++c) {
    const qsv_circuit_rec& r = cr[c];
    if (r.n <= CB_SMEM_QUBITS) continue;
    segidx[(size_t)c].x = (int)segs.size();
    int64_t i = r.gate_offset;
    const int64_t end = r.gate_offset + r.ngates;
    do {
      uint32_t set = 0x1Fu;  // address bits 0..4 stay local (coalesced chunk accesses)
      int64_t j = i;
      for (; j < end; ++j) {
        const qsv_gate_rec& g = gv[(size_t)j];
        const int need = g.kind == G_CX ? 2 : (g.kind == G_CSWAP ? 3 : 1);
        const int qs[3] = {g.q0, g.q1, g.q2};
        uint32_t gm = 0;
        for (int t = 0; t < need; ++t) gm |= 1u << (r.n - 1 - qs[t]);
        if (__builtin_popcount(set | gm) > CB_SMEM_QUBITS) break;
        set |= gm;
      }
      for (int p = 0; p < r.n && __builtin_popcount(set) < CB_SMEM_QUBITS; ++p) set |= 1u << p;
      SegmentRec sg;
      sg.gate_begin = (int32_t)i;
      sg.gate_end = (int32_t)j;
      int local_of[32];
      for (int p = 0, li = 0; p < r.n; ++p)
        if ((set >> p) & 1u) {
          sg.lpos[li] = p;
          local_of[p] = li++;
        }
      for (int64_t k = i; k < j; ++k) {
        qsv_gate_rec& g = gv[(size_t)k];
        const int need = g.kind == G_CX ? 2 : (g.kind == G_CSWAP ? 3 : 1);
        int* qs[3] = {&g.q0, &g.q1, &g.q2};
        for (int t = 0; t < need; ++t) *qs[t] = CB_SMEM_QUBITS - 1 - local_of[r.n - 1 - *qs[t]];
      }
      segs.push_back(sg);
      i = j;
    } while (i < end);
    segidx[(size_t)c].y = (int)segs.size();
  }
  auto* b = new (std::nothrow) qsv_circuits();
  if (!b) return set_error(nullptr, QSV_ERR_OOM, "host allocation failed");
  b->ncirc = ncirc;
  b->state_amps = amps;
  // Cluster size and the leading circuits that run on a whole cluster (n large enough to
  // give every CTA of the cluster at least one chunk per segment).
  // 6: config 4's list (4096 circuits, n ~ U[8,20]) measured 105 K circuits/s with
  // p99/p50 latency 18.6, against 116 K / 26.9 at 4, 97 K / 13.6 at 8 and 126 K / 105
  // without clusters (clusters of 4 or 6 fill 144 of 152 SMs, of 8 only 120).
  b->cluster = 6;
  if (const char* env = getenv("QSV_CIRCUIT_CLUSTER")) {
    const int v = atoi(env);
    if (v >= 1 && v <= 8) b->cluster = v;
  }
  int min_n = CB_SMEM_QUBITS + 1;
  while ((1 << (min_n - CB_SMEM_QUBITS)) < 2 * b->cluster) ++min_n;
  if (b->cluster > 1)
    while (b->nbig < ncirc && cr[b->nbig].n >= min_n) ++b->nbig;
  b->h_circs.assign(cr, cr + ncirc);
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, dev);
  bool ok = cudaMalloc(&b->d_gates, std::max<int64_t>(1, ngates) * sizeof(qsv_gate_rec)) == cudaSuccess &&
            cudaMalloc(&b->d_circs, ncirc * sizeof(qsv_circuit_rec)) == cudaSuccess &&
            cudaMalloc(&b->d_feeds, std::max<int64_t>(1, nfeeds) * sizeof(float2)) == cudaSuccess &&
            cudaMalloc(&b->d_states, amps * sizeof(float2)) == cudaSuccess &&
            cudaMalloc(&b->d_times, 2 * (size_t)ncirc * sizeof(unsigned long long)) == cudaSuccess &&
            cudaMalloc(&b->d_counter, 2 * sizeof(int)) == cudaSuccess &&
            cudaMalloc(&b->d_segs, std::max<size_t>(1, segs.size()) * sizeof(SegmentRec)) == cudaSuccess &&
            cudaMalloc(&b->d_segidx, (size_t)ncirc * sizeof(int2)) == cudaSuccess;
  if (ok)
    ok = cudaMemcpy(b->d_gates, gv.data(), ngates * sizeof(qsv_gate_rec), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(b->d_segidx, segidx.data(), (size_t)ncirc * sizeof(int2), cudaMemcpyHostToDevice) ==
             cudaSuccess &&
         (segs.empty() || cudaMemcpy(b->d_segs, segs.data(), segs.size() * sizeof(SegmentRec),
                                     cudaMemcpyHostToDevice) == cudaSuccess) &&
         cudaMemcpy(b->d_circs, circuits, ncirc * sizeof(qsv_circuit_rec), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(b->d_feeds, feeds, nfeeds * sizeof(float2), cudaMemcpyHostToDevice) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    qsv_circuits_destroy(b);
    return set_error(nullptr, QSV_ERR_OOM, "circuit batch allocation/upload failed");
  }
  *out = b;
  return QSV_OK;
}

int qsv_circuits_run(qsv_circuits* b, void* stream) {
  if (!b) return set_error(nullptr, QSV_ERR_INVALID, "null batch");
  cudaStream_t st = (cudaStream_t)stream;
  if (b->graph && b->graph_stream != st) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  if (!b->graph) {
    if (!st) return set_error(nullptr, QSV_ERR_INVALID, "a non-default stream is needed to capture the launch");
    int rc = capture(b, st);
    if (rc) return rc;
  }
  cudaError_t e = cudaGraphLaunch(b->graph, st);
  if (e != cudaSuccess) return set_error(nullptr, QSV_ERR_CUDA, "graph launch: %s", cudaGetErrorString(e));
  count_launch();
  return QSV_OK;
}

int qsv_circuits_read(qsv_circuits* b, int circuit, void* host_out) {
  if (!b || !host_out || circuit < 0 || circuit >= b->ncirc) return set_error(nullptr, QSV_ERR_INVALID, "bad read");
  const qsv_circuit_rec& r = b->h_circs[(size_t)circuit];
  cudaError_t e = cudaMemcpy(host_out, b->d_states + r.state_offset, (sizeof(float2) << r.n), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return set_error(nullptr, QSV_ERR_CUDA, "read: %s", cudaGetErrorString(e));
  return QSV_OK;
}

int qsv_circuits_times(qsv_circuits* b, unsigned long long* host_out) {
  if (!b || !host_out) return set_error(nullptr, QSV_ERR_INVALID, "bad read");
  cudaError_t e = cudaMemcpy(host_out, b->d_times, 2 * (size_t)b->ncirc * sizeof(unsigned long long),
                             cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return set_error(nullptr, QSV_ERR_CUDA, "times: %s", cudaGetErrorString(e));
  return QSV_OK;
}

int qsv_circuits_destroy(qsv_circuits* b) {
  if (!b) return QSV_OK;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  cudaFree(b->d_gates);
  cudaFree(b->d_circs);
  cudaFree(b->d_feeds);
  cudaFree(b->d_states);
  cudaFree(b->d_times);
  cudaFree(b->d_counter);
  cudaFree(b->d_segs);
  cudaFree(b->d_segidx);
  delete b;
  return QSV_OK;
}

}  // extern "C"
