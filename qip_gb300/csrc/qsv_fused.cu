// Fused dense blocks on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// A fused block is a 2^k x 2^k complex matrix U (4 <= k <= 6) on k target qubits, the
// product of a run of gates that only touch those qubits.  It is applied to every one
// of the 2^(n-k) amplitude groups of a complex64 state in one HBM pass.
//
// GEMM shape.  A CTA tile holds 128 groups ("batch" b, the 7 lowest non-target bits)
// x 2^k target combinations.  Writing v_b in R^(2^(k+1)) as [Re; Im], the block is the
// real matrix W = [[Ur, -Ui], [Ui, Ur]] (KD x KD, KD = 2^(k+1)) and the tile update is
//     D[b][n] = sum_kk A[b][kk] * W[n][kk]      (M = 128, N = K = KD)
// with A the tile (row b = v_b).  D row b then holds [Re w_b; Im w_b] in one TMEM
// lane, so each epilogue thread writes whole output amplitudes and a warp writes 32
// consecutive groups: coalesced stores without a shuffle.
//
// Precision.  Operands are split into bf16 pairs x = hi + lo (hi = bf16(x),
// lo = bf16(x - hi)) and D accumulates hi*hi + hi*lo + lo*hi in FP32 (three
// tcgen05.mma kind::f16 passes), about 2^-16 relative error per pass.
//
// Shared-memory operands use the canonical K-major layout without swizzle: core
// matrices of 8 rows x 16 bytes; the leading byte offset (LBO) steps along K between
// core matrices and the stride byte offset (SBO = 128 B) steps between 8-row groups.
// A row r, element kk lives at (kk/8)*(rows*16) + r*16 + (kk%8)*2.
//
// Every wait is bounded: a stuck mbarrier sets the handle's status word and the kernel
// still frees its tensor memory before returning.

#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "qsv_internal.cuh"
#include "qsv_tc.cuh"

using namespace qsv;

namespace {

constexpr int FB_M = 128;         // groups per tile (MMA M)
constexpr int FB_THREADS = 256;   // 8 warps
constexpr int FB_BATCH_BITS = 7;  // log2(FB_M)

template <int KQ>
struct FB {
  static constexpr int T = 1 << KQ;            // target combinations
  static constexpr int KD = 2 * T;             // GEMM K = N
  static constexpr int EBITS = FB_BATCH_BITS + KQ;  // bits of the tile index
  static constexpr int TILE = FB_M * T;        // amplitudes per tile
  static constexpr int A_BYTES = FB_M * KD * 2;  // one bf16 copy of the tile
  static constexpr int W_BYTES = KD * KD * 2;    // one bf16 copy of W
  static constexpr int RAW_BYTES = TILE * 8;     // complex64 staging of one tile
  static constexpr int A_LBO = FB_M * 16;        // K-step between core matrices of A
  static constexpr int W_LBO = KD * 16;
  static constexpr int VEC = TILE / 2 / FB_THREADS;             // float4 (2 amplitudes) per thread
  static constexpr int ITEMS = (FB_M * (T / 8)) / FB_THREADS;  // (b, 8 targets) per thread
  static constexpr int TMEM_COLS = KD < 32 ? 32 : KD;       // one accumulator
  static constexpr int TMEM_COLS2 = 2 * KD < 32 ? 32 : 2 * KD;  // two (shuffle mode)
  static constexpr int COLS_PER_WARP = T / 2;  // output targets handled per warp
  // Tables: eb[128] u16, et[T] u16, swz[TILE/16] u8, dephi[T] u64; then the mbarrier.
  static constexpr int TAB_BYTES = FB_M * 2 + T * 2 + TILE / 16 + T * 8;
  static constexpr int SMEM = 2 * A_BYTES + 2 * W_BYTES + RAW_BYTES + ((TAB_BYTES + 15) / 16) * 16 + 64;
  // The direct variant stages nothing: no RAW buffer.
  static constexpr int SMEM_DIRECT = SMEM - RAW_BYTES;
};

// Tile geometry.  A tile covers the 2^k target combinations t and 128 groups b (the
// 7 lowest non-target bit positions).  Its 7+k bit positions, sorted, are P; tile
// element e (bit i of e <-> position P[i]) lives at tile_base + dep(e).  P always starts
// with positions 0..6, so dep(e) = (e & 127) + dephi[e >> 7] and 16-byte pairs of
// consecutive e are adjacent amplitudes.  The shared staging buffer stores element e at
// word e ^ (swz[e >> 4] << 1): a host-chosen XOR of 16-byte slots that keeps the
// (b-consecutive) transposing accesses spread over the banks for any placement.
//
// Shuffle mode (for targets among address bits 0..4 that are not a prefix): lane x of a
// warp always loads and stores address bit pattern x of 32 consecutive amplitudes.
// Kernel target order t' lists the targets by ascending position (the block matrix is
// permuted to match, tperm), so the j targets in bits 0..4 are t' bits 0..j-1.  After
// the load, up to three exchange rounds (shfl.xor on lane bit = that target's address
// bit, register bit i) move t' bits 0..2 into register bits 0..2: each group of 8
// registers then holds one row m and 8 consecutive t' of the A operand.  The epilogue
// reads TMEM row m = 32*(warp%4) + lane, columns t' = (warp/4)*T/2 + c, and j exchange
// rounds (lane bits whose group bit is above address bit 4 <-> c bits 0..j-1) restore
// 32 consecutive amplitudes per store.  All addresses and operand offsets are sums of
// per-bit contributions listed in the tables below.
//
// Prefix mode (6-qubit blocks whose targets include address bits 0, 1 and 2, so 8
// consecutive t are adjacent amplitudes): the products run transposed, D^T = W A^T (W in
// the MMA's A slot with its rows interleaved [Re t, Im t], the tile in the B slot), so
// TMEM lane 2t / 2t+1 holds Re / Im of output target t and column b holds group b.  A
// warp's lanes then cover 16 consecutive targets of one group: after one shfl.xor that
// pairs Re with Im, each store instruction writes two whole 128-byte runs (groups b and
// b+1), where the direct epilogue (one group per lane) would touch 32 lines.  Loads take
// 32-byte runs of 4 targets, 4 lanes per 128-byte line and 8 groups per warp.
constexpr int MODE_DIRECT = 0;
constexpr int MODE_STAGED = 1;
constexpr int MODE_SHUF = 2;
constexpr int MODE_PREFIX = 3;
// Pair modes (6-qubit blocks whose lowest targets are a run of 4 on address bits m..m+3
// above m = 1 or 2 group bits): the prefix mode's transposed products and epilogue (each
// store instruction then writes one run of 32 (m = 1) or two half-sector runs (m = 2)),
// with loads of 32-byte runs that hold 2 groups x 2 targets (m = 1) or 4 groups x 1
// target (m = 2), turned into runs of 4 targets of one group by lane exchanges: a
// register swap and one shfl.xor round (m = 1) or a 4 x 4 transpose (m = 2).
constexpr int MODE_PAIR1 = 4;
constexpr int MODE_PAIR2 = 5;
constexpr int NUM_MODES = 6;

struct BlockArgs {
  uint64_t ntiles;
  int k;
  int mode;             // MODE_DIRECT, MODE_STAGED or MODE_SHUF
  int vec;              // direct: amplitudes per global access (1, 2 or 4): t's lowest bits are
                        // the target bits 0.. of the address, so t..t+vec-1 are adjacent
  int ptile[16];        // the 7+k tile positions, ascending (zero insertion -> tile base)
  uint16_t eb[FB_M];    // e of group b
  uint16_t et[64];      // e of target combination t (targets[0] = MSB of t)
  uint8_t swz[512];     // 3-bit slot swizzle per (e >> 4)
  uint64_t dephi[64];   // address offset of e >> 7
  // Shuffle mode tables (see above).
  int nld, nst;         // exchange rounds after the load / in the epilogue
  int ld_lane[3];       // lane bit of load round i (register bit i)
  int st_lane[5];       // lane bit of epilogue round i (register bit i)
  uint64_t ld_warp[3];  // address contribution of warp bits (lane x contributes x)
  uint64_t ld_reg[32];  // address offset of load register r
  uint32_t a_lw[8];     // A byte offset of lane bits 0..4 and warp bits 0..2 after the load rounds
  uint32_t a_it[4];     // A byte offset of register group it (registers 8*it .. 8*it+7)
  uint64_t st_lw[8];    // address contribution of lane bits 0..4, warp bits 0..1 (row quadrant), warp bit 2
  uint64_t st_reg[32];  // address offset of epilogue register c
  uint8_t tperm[64];    // kernel target order t' -> the caller's block matrix index
  const uint4* wimg;    // hi image then lo image (2 * W_BYTES bytes)
  int* flag;            // status word
  uint64_t wait_ns;     // limit of each wait for a tile's products
  int stall_first;      // fault injection: the first such wait is on a barrier nothing arrives on
  // Batches (the tensor-core adjoint): psi holds several states of set_amps amplitudes,
  // each with its own matrix; state s's image is at wimg + s * img_stride bytes.  Tiles
  // are numbered state by state, set_tiles per state (a power of two); 0: one state.
  uint64_t set_tiles;
  uint64_t set_amps;
  uint64_t img_stride;
  int reverse;          // visit the tiles from the last one down (one state only)
};

// MODE_DIRECT: each thread loads (b, 8 targets) items straight from global memory and
// the epilogue stores TMEM rows straight back; coalesced when the 5 lowest address bits
// are batch bits (or the low targets are an address prefix, vec > 1).  MODE_STAGED: the
// tile moves through a shared staging buffer in address order (16-byte coalesced global
// accesses for any placement) at the cost of two extra shared-memory passes.
// MODE_SHUF: lane = 5 lowest address bits, warp shuffles transpose in registers.
template <int KQ, int MODE>
__global__ void __launch_bounds__(FB_THREADS, 1)
    k_block_tc(float2* __restrict__ psi, const __grid_constant__ BlockArgs a) {
  using P = FB<KQ>;
  constexpr bool STAGED = MODE == MODE_STAGED;
  constexpr bool SHUF = MODE == MODE_SHUF;
  constexpr bool PREFIX = MODE == MODE_PREFIX;
  constexpr int PAIR = MODE == MODE_PAIR1 ? 1 : (MODE == MODE_PAIR2 ? 2 : 0);  // group bits below the targets
  constexpr bool TRANS = PREFIX || PAIR > 0;  // transposed products and epilogue
  static_assert(!TRANS || KQ == 6, "the prefix and pair modes are built for 6-qubit blocks");
  constexpr int SMEM_USED = STAGED ? P::SMEM : P::SMEM_DIRECT;
  constexpr int RAW = STAGED ? P::RAW_BYTES : 0;
  constexpr int R = P::T / 2;  // shuffle mode: amplitudes per thread
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sA_hi = smem;
  uint8_t* sA_lo = smem + P::A_BYTES;
  uint8_t* sW_hi = smem + 2 * P::A_BYTES;
  uint8_t* sW_lo = sW_hi + P::W_BYTES;
  float2* raw = reinterpret_cast<float2*>(sW_lo + P::W_BYTES);
  float4* raw4 = reinterpret_cast<float4*>(raw);
  uint16_t* eb = reinterpret_cast<uint16_t*>(sW_lo + P::W_BYTES + RAW);
  uint16_t* et = eb + FB_M;
  uint8_t* swz = reinterpret_cast<uint8_t*>(et + P::T);
  uint64_t* dephi = reinterpret_cast<uint64_t*>(swz + P::TILE / 16);
  // Tail: two mbarriers (one per accumulator), the TMEM address, the abort flag, and
  // the barrier of the injected stall (initialised, never arrived on).
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + SMEM_USED - 64);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mbar + 2);
  int* abort_flag = reinterpret_cast<int*>(tmem_slot + 1);
  uint64_t* stall_bar = mbar + 3;
  constexpr int TCOLS = SHUF ? P::TMEM_COLS2 : P::TMEM_COLS;

  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const int lane = tid & 31;

  // W image (hi then lo) and the geometry tables into shared memory.  In a batch the
  // image is that of the state the CTA's current tile belongs to (reloaded below when a
  // tile of another state comes up, with no products in flight).
  const int set_shift = a.set_tiles ? __ffsll((long long)a.set_tiles) - 1 : 0;
  auto set_of = [&](uint64_t t) -> uint64_t { return a.set_tiles ? (t >> set_shift) : 0ull; };
  auto load_w = [&](uint64_t set) {
    const uint4* src = reinterpret_cast<const uint4*>(reinterpret_cast<const uint8_t*>(a.wimg) + set * a.img_stride);
    uint4* dst = reinterpret_cast<uint4*>(sW_hi);
    constexpr int NV = (2 * P::W_BYTES) / 16;
    for (int i = tid; i < NV; i += FB_THREADS) dst[i] = src[i];
  };
  uint64_t cur_set = set_of(blockIdx.x);
  load_w(cur_set);
  for (int i = tid; i < FB_M; i += FB_THREADS) eb[i] = a.eb[i];
  for (int i = tid; i < P::T; i += FB_THREADS) {
    et[i] = a.et[i];
    dephi[i] = a.dephi[i];
  }
  for (int i = tid; i < P::TILE / 16; i += FB_THREADS) swz[i] = a.swz[i];
  if (tid == 0) {
    mbar_init(smem_u32(mbar), 1);
    mbar_init(smem_u32(mbar + 1), 1);
    mbar_init(smem_u32(stall_bar), 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"((uint32_t)TCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  auto bar_of = [&](int s) -> uint32_t { return smem_u32(mbar + s); };
  constexpr uint32_t idesc = make_idesc(FB_M, P::KD);

  auto slot = [&](int e) -> int { return e ^ ((int)swz[e >> 4] << 1); };
  auto dep = [&](int e) -> uint64_t { return (uint64_t)(e & (FB_M - 1)) + dephi[e >> FB_BATCH_BITS]; };
  // Item it of this thread: group b and target chunk tg (targets tg*8 .. tg*8+7); lanes
  // take consecutive groups.
  auto item_b = [&](int it) -> int { return (it * FB_THREADS + tid) & (FB_M - 1); };
  auto item_tg = [&](int it) -> int { return (it * FB_THREADS + tid) >> FB_BATCH_BITS; };
  // Prefix mode: quarter-items of 4 targets (one 32-byte load).  Quarter u of this thread
  // is group ((warp*8 + lane/4) | (u&1)*64), targets 4*q4 .. 4*q4+3 with
  // q4 = (lane&3) | (u>>1)*4: four lanes read one 128-byte run of a group (8 whole lines
  // per warp load), and the 8-byte operand stores of a warp fill 16 distinct bank slots.
  auto quarter_b = [&](int u) -> int { return ((warp << 3) | (lane >> 2)) | ((u & 1) << 6); };
  auto quarter_t4 = [&](int u) -> int { return (lane & 3) | ((u >> 1) << 2); };
  // Pair modes: load u of this thread starts at group pair_lb(u), target pair_lt(u) (the
  // run's other amplitudes differ in the group bits below the targets, and for m = 1 in
  // target bit 0); after the exchanges the thread holds group pair_b(u), targets
  // 4*pair_q4(u) .. +3.  With l = lane bits, w = warp:
  //   m = 1: loads t bits 1, 2, 3 = l0, l1, l2; b bits 1, 2 = l3, l4; b bits 3..5 = w;
  //          t bits 4, 5 = u bits 0, 1; b bit 6 = u bit 2.  Held: b bit 0 = l0.
  //   m = 2: loads t bits 0, 1, 2 = l0, l1, l2; b bits 2, 3 = l3, l4; b bits 4..6 = w;
  //          t bits 3..5 = u.  Held: b bits 0, 1 = l0, l1.
  auto lb = [&](int i) -> int { return (lane >> i) & 1; };
  auto pair_lb = [&](int u) -> int {
    return PAIR == 1 ? (lb(3) << 1) | (lb(4) << 2) | (warp << 3) | ((u >> 2) << 6) : (lb(3) << 2) | (lb(4) << 3) | (warp << 4);
  };
  auto pair_lt = [&](int u) -> int {
    return PAIR == 1 ? (lb(0) << 1) | (lb(1) << 2) | (lb(2) << 3) | ((u & 3) << 4) : lb(0) | (lb(1) << 1) | (lb(2) << 2) | (u << 3);
  };
  auto pair_b = [&](int u) -> int {
    return PAIR == 1 ? lb(0) | (lb(3) << 1) | (lb(4) << 2) | (warp << 3) | ((u >> 2) << 6)
                     : lb(0) | (lb(1) << 1) | (lb(3) << 2) | (lb(4) << 3) | (warp << 4);
  };
  auto pair_q4 = [&](int u) -> int { return PAIR == 1 ? lb(1) | (lb(2) << 1) | ((u & 3) << 2) : lb(2) | (u << 1); };

  // Staged: thread u-th pair holds elements e, e+1 with e = 2*(u*256 + tid) (adjacent
  // amplitudes).  Direct: item it holds (b, targets tg*8..tg*8+7).
  float4 buf[P::VEC];
  float2 buf2[P::ITEMS][8];
  float2 v[SHUF ? R : 1];
  // Shuffle mode: per-thread sums of the lane/warp contributions.
  uint64_t ld_lw = 0, st_lw = 0;
  uint32_t a_lw = 0;
  if constexpr (SHUF) {
    ld_lw = (uint64_t)lane;
#pragma unroll
    for (int i = 0; i < 3; ++i)
      if ((warp >> i) & 1) ld_lw += a.ld_warp[i];
#pragma unroll
    for (int i = 0; i < 5; ++i)
      if ((lane >> i) & 1) {
        a_lw += a.a_lw[i];
        st_lw += a.st_lw[i];
      }
#pragma unroll
    for (int i = 0; i < 3; ++i)
      if ((warp >> i) & 1) {
        a_lw += a.a_lw[5 + i];
        st_lw += a.st_lw[5 + i];
      }
  }
  [[maybe_unused]] const uint64_t lim = a.ntiles * (uint64_t)P::TILE;  // the state's size
  auto load_tile = [&](uint64_t base) {
    if constexpr (SHUF) {
      const float2* src = psi + base + ld_lw;
#pragma unroll
      for (int r = 0; r < R; ++r)
        v[r] = QSV_IN_BOUNDS(base + ld_lw + a.ld_reg[r], lim) ? __ldcs(src + a.ld_reg[r]) : make_float2(0.f, 0.f);
    } else if constexpr (STAGED) {
#pragma unroll
      for (int u = 0; u < P::VEC; ++u) {
        const int e = 2 * (u * FB_THREADS + tid);
        if (QSV_IN_BOUNDS(base + dep(e) + 1, lim)) buf[u] = __ldcs(reinterpret_cast<const float4*>(psi + base + dep(e)));
      }
    } else if constexpr (PREFIX) {
#pragma unroll
      for (int u = 0; u < 2 * P::ITEMS; ++u) {
        const uint64_t off = base + dep(eb[quarter_b(u)]) + dep(et[4 * quarter_t4(u)]);
        if (QSV_IN_BOUNDS(off + 3, lim)) ld_v8(psi + off, &buf2[u >> 1][(u & 1) * 4]);
      }
    } else if constexpr (PAIR > 0) {
#pragma unroll
      for (int u = 0; u < 2 * P::ITEMS; ++u) {
        const uint64_t off = base + dep(eb[pair_lb(u)]) + dep(et[pair_lt(u)]);
        if (QSV_IN_BOUNDS(off + 3, lim)) ld_v8(psi + off, &buf2[u >> 1][(u & 1) * 4]);
      }
    } else if (a.vec == 4) {
#pragma unroll
      for (int it = 0; it < P::ITEMS; ++it) {
        const int b = item_b(it);
        const int tg = item_tg(it);
        const uint64_t rb = base + dep(eb[b]);
#pragma unroll
        for (int j = 0; j < 8; j += 4)
          if (QSV_IN_BOUNDS(rb + dep(et[tg * 8 + j]) + 3, lim)) ld_v8(psi + rb + dep(et[tg * 8 + j]), &buf2[it][j]);
      }
    } else if (a.vec == 2) {
#pragma unroll
      for (int it = 0; it < P::ITEMS; ++it) {
        const int item = it * FB_THREADS + tid;
        const int b = item & (FB_M - 1);
        const int tg = item >> FB_BATCH_BITS;
        const uint64_t rb = base + dep(eb[b]);
#pragma unroll
        for (int j = 0; j < 8; j += 2) {
          if (!QSV_IN_BOUNDS(rb + dep(et[tg * 8 + j]) + 1, lim)) continue;
          const float4 v = __ldcs(reinterpret_cast<const float4*>(psi + rb + dep(et[tg * 8 + j])));
          buf2[it][j] = make_float2(v.x, v.y);
          buf2[it][j + 1] = make_float2(v.z, v.w);
        }
      }
    } else {
#pragma unroll
      for (int it = 0; it < P::ITEMS; ++it) {
        const int item = it * FB_THREADS + tid;
        const int b = item & (FB_M - 1);
        const int tg = item >> FB_BATCH_BITS;
        const uint64_t rb = base + dep(eb[b]);
#pragma unroll
        for (int j = 0; j < 8; ++j)
          if (QSV_IN_BOUNDS(rb + dep(et[tg * 8 + j]), lim)) buf2[it][j] = __ldcs(&psi[rb + dep(et[tg * 8 + j])]);
      }
    }
  };

  // Tile i of this CTA accumulates in TMEM columns [acc(i), acc(i) + KD).  The shuffle
  // mode alternates two accumulators: the products of tile i run while the epilogue of
  // tile i-1 drains the other one, and the only wait per tile is for the products of
  // tile i-1 (issued a whole iteration earlier) before A is rewritten; that hides the
  // products behind its heavier epilogue.  The direct and staged modes keep one
  // accumulator and wait for the products right after prefetching the next tile: the
  // wait gives those loads a head start, which matters more to them (measured: the
  // direct mode is bound by loads in flight, not by the serial chain), and the staged
  // mode shares its staging buffer between the operand and the epilogue.
  auto write_a = [&]() {
      // 1. Stage the tile in address order.
      if constexpr (STAGED) {
  #pragma unroll
        for (int u = 0; u < P::VEC; ++u) {
          const int e = 2 * (u * FB_THREADS + tid);
          raw4[slot(e) >> 1] = buf[u];
        }
        __syncthreads();
      }
      // 2. Transpose into the A operand: row b, K = [Re t | Im t], bf16 hi/lo split.
      if constexpr (SHUF) {
  #pragma unroll
        for (int i = 0; i < 3; ++i) {
          if (i < a.nld) {
            const int lb = a.ld_lane[i];
            const bool up = (lane >> lb) & 1;
  #pragma unroll
            for (int r = 0; r < R; ++r) {
              if (r & (1 << i)) continue;
              const int r1 = r | (1 << i);
              const float2 send = up ? v[r] : v[r1];
              float2 got;
              got.x = __shfl_xor_sync(0xffffffffu, send.x, 1 << lb);
              got.y = __shfl_xor_sync(0xffffffffu, send.y, 1 << lb);
              if (up)
                v[r] = got;
              else
                v[r1] = got;
            }
          }
        }
  #pragma unroll
        for (int it = 0; it < R / 8; ++it) {
          float re[8], im[8];
  #pragma unroll
          for (int g = 0; g < 8; ++g) {
            re[g] = v[8 * it + g].x;
            im[g] = v[8 * it + g].y;
          }
          uint4 rh, rl, ih, il;
          split8(re, rh, rl);
          split8(im, ih, il);
          const uint32_t off_re = a_lw + a.a_it[it];
          const uint32_t off_im = off_re + (P::T / 8) * P::A_LBO;
          *reinterpret_cast<uint4*>(sA_hi + off_re) = rh;
          *reinterpret_cast<uint4*>(sA_lo + off_re) = rl;
          *reinterpret_cast<uint4*>(sA_hi + off_im) = ih;
          *reinterpret_cast<uint4*>(sA_lo + off_im) = il;
        }
      }
      if constexpr (PAIR == 1) {
        // Register bit 0 = group bit 0, bit 1 = target bit 0: swap them, then trade
        // register bit 1 (group bit 0) for lane bit 0 (target bit 1).
        const bool up = lane & 1;
  #pragma unroll
        for (int u = 0; u < 2 * P::ITEMS; ++u) {
          float2* r = &buf2[u >> 1][(u & 1) * 4];
          const float2 x = r[1];
          r[1] = r[2];
          r[2] = x;
  #pragma unroll
          for (int j = 0; j < 2; ++j) {
            const float2 send = up ? r[j] : r[j + 2];
            float2 got;
            got.x = __shfl_xor_sync(0xffffffffu, send.x, 1);
            got.y = __shfl_xor_sync(0xffffffffu, send.y, 1);
            if (up)
              r[j] = got;
            else
              r[j + 2] = got;
          }
        }
      } else if constexpr (PAIR == 2) {
        // Register bits 0, 1 = group bits 0, 1; lane bits 0, 1 = target bits 0, 1:
        // transpose the 4 x 4 blocks (two shfl.xor rounds).
  #pragma unroll
        for (int bb = 0; bb < 2; ++bb) {
          const bool up = (lane >> bb) & 1;
  #pragma unroll
          for (int u = 0; u < 2 * P::ITEMS; ++u) {
            float2* r = &buf2[u >> 1][(u & 1) * 4];
  #pragma unroll
            for (int j = 0; j < 4; ++j) {
              if (j & (1 << bb)) continue;
              const int j1 = j | (1 << bb);
              const float2 send = up ? r[j] : r[j1];
              float2 got;
              got.x = __shfl_xor_sync(0xffffffffu, send.x, 1 << bb);
              got.y = __shfl_xor_sync(0xffffffffu, send.y, 1 << bb);
              if (up)
                r[j] = got;
              else
                r[j1] = got;
            }
          }
        }
      }
      if constexpr (TRANS) {
  #pragma unroll
        for (int u = 0; u < 2 * P::ITEMS; ++u) {
          const int b = PAIR ? pair_b(u) : quarter_b(u), q4 = PAIR ? pair_q4(u) : quarter_t4(u);
          float re[4], im[4];
  #pragma unroll
          for (int j = 0; j < 4; ++j) {
            re[j] = buf2[u >> 1][(u & 1) * 4 + j].x;
            im[j] = buf2[u >> 1][(u & 1) * 4 + j].y;
          }
          uint2 rh, rl, ih, il;
          split4(re, rh, rl);
          split4(im, ih, il);
          const int off_re = (q4 >> 1) * P::A_LBO + b * 16 + (q4 & 1) * 8;
          const int off_im = off_re + (P::T / 8) * P::A_LBO;
          *reinterpret_cast<uint2*>(sA_hi + off_re) = rh;
          *reinterpret_cast<uint2*>(sA_lo + off_re) = rl;
          *reinterpret_cast<uint2*>(sA_hi + off_im) = ih;
          *reinterpret_cast<uint2*>(sA_lo + off_im) = il;
        }
      }
  #pragma unroll
      for (int it = 0; it < ((SHUF || TRANS) ? 0 : P::ITEMS); ++it) {
        const int b = item_b(it);
        const int tg = item_tg(it);
        const int eb_ = eb[b];
        float re[8], im[8];
  #pragma unroll
        for (int j = 0; j < 8; ++j) {
          const float2 v = STAGED ? raw[slot(eb_ | et[tg * 8 + j])] : buf2[it][j];
          re[j] = v.x;
          im[j] = v.y;
        }
        uint4 rh, rl, ih, il;
        split8(re, rh, rl);
        split8(im, ih, il);
        const int off_re = tg * P::A_LBO + b * 16;
        const int off_im = (P::T / 8 + tg) * P::A_LBO + b * 16;
        *reinterpret_cast<uint4*>(sA_hi + off_re) = rh;
        *reinterpret_cast<uint4*>(sA_lo + off_re) = rl;
        *reinterpret_cast<uint4*>(sA_hi + off_im) = ih;
        *reinterpret_cast<uint4*>(sA_lo + off_im) = il;
      }
  };
  auto issue_mma = [&](uint32_t acc, uint32_t barrier) {
    if (tid == 0) {
      const uint32_t a_hi = smem_u32(sA_hi), a_lo = smem_u32(sA_lo);
      const uint32_t w_hi = smem_u32(sW_hi), w_lo = smem_u32(sW_lo);
      constexpr int KSTEPS = P::KD / 16;
      // The two small correction passes first, the main pass last: each accumulation
      // rounds relative to the accumulator's current size, so the corrections' roundings
      // stay at their own (2^-8 smaller) scale and only the main pass's 8 adds round at
      // full scale (against 24 the other way round; the FP32 accumulation rounds towards
      // zero, which otherwise shrinks the norm by ~1.5e-6 per block).  The prefix mode
      // multiplies transposed: W in the first operand slot (M = KD = 128 rows), the
      // tile in the second (N = 128 groups); the instruction descriptor is the same.
      auto mma = [&](uint32_t tile_img, uint32_t w_img, int s, uint32_t accumulate) {
        const uint64_t td = make_smem_desc(tile_img + s * 2 * P::A_LBO, P::A_LBO, 128);
        const uint64_t wd = make_smem_desc(w_img + s * 2 * P::W_LBO, P::W_LBO, 128);
        if constexpr (TRANS)
          tc_mma(acc, wd, td, idesc, accumulate);
        else
          tc_mma(acc, td, wd, idesc, accumulate);
      };
#pragma unroll
      for (int s = 0; s < KSTEPS; ++s) mma(a_hi, w_lo, s, s > 0 ? 1u : 0u);
#pragma unroll
      for (int s = 0; s < KSTEPS; ++s) mma(a_lo, w_hi, s, 1u);
#pragma unroll
      for (int s = 0; s < KSTEPS; ++s) mma(a_hi, w_hi, s, 1u);
      tc_commit(barrier);
    }
  };
  auto epilogue = [&](uint64_t tbase, uint32_t acc) {
      // 5. Epilogue: TMEM lane b -> the staging buffer.  Warp w reads lanes 32*(w%4)..
      //    and output targets [h*T/2, (h+1)*T/2) with h = w/4.
      if constexpr (SHUF) {
        constexpr int CHS = P::COLS_PER_WARP;
        const int q = warp & 3;
        const int h = warp >> 2;
        const uint32_t lane_addr = acc + ((uint32_t)(q * 32) << 16);
        float re[CHS], im[CHS];
        tmem_ld<CHS>(lane_addr + (uint32_t)(h * CHS), re);
        tmem_ld<CHS>(lane_addr + (uint32_t)(P::T + h * CHS), im);
        tmem_ld_wait();
  #pragma unroll
        for (int i = 0; i < 5; ++i) {
          if (i < KQ - 1 && i < a.nst) {
            const int lb = a.st_lane[i];
            const bool up = (lane >> lb) & 1;
  #pragma unroll
            for (int c = 0; c < CHS; ++c) {
              if (c & (1 << i)) continue;
              const int c1 = c | (1 << i);
              const float sr = up ? re[c] : re[c1];
              const float si = up ? im[c] : im[c1];
              const float gr = __shfl_xor_sync(0xffffffffu, sr, 1 << lb);
              const float gi = __shfl_xor_sync(0xffffffffu, si, 1 << lb);
              if (up) {
                re[c] = gr;
                im[c] = gi;
              } else {
                re[c1] = gr;
                im[c1] = gi;
              }
            }
          }
        }
        float2* dst = psi + tbase + st_lw;
  #pragma unroll
        for (int c = 0; c < CHS; ++c)
          if (QSV_IN_BOUNDS(tbase + st_lw + a.st_reg[c], lim)) __stcs(dst + a.st_reg[c], make_float2(re[c], im[c]));
      } else if constexpr (TRANS) {
        // Lane row 32q + lane = component (lane & 1) of target t; warp half h reads
        // groups 64h .. 64h+63.  Pairs of lanes swap halves: the even lane keeps group
        // b and the odd lane group b+1, each with its (Re, Im).
        const int q = warp & 3;
        const int h = warp >> 2;
        const bool odd = lane & 1;
        const uint64_t ot = dep(et[(q * 32 + lane) >> 1]);
        const uint32_t lane_addr = acc + ((uint32_t)(q * 32) << 16);
  #pragma unroll
        for (int c0 = 0; c0 < 64; c0 += 32) {
          float col[32];
          tmem_ld<32>(lane_addr + (uint32_t)(h * 64 + c0), col);
          tmem_ld_wait();
          if constexpr (PAIR == 2) {
            // Groups b..b+3 are address bits 0, 1: the even lane takes b, b+1 and the odd
            // lane b+2, b+3, each one 16-byte store (a lane pair fills a 32-byte sector).
  #pragma unroll
            for (int i = 0; i < 32; i += 4) {
              const float g0 = __shfl_xor_sync(0xffffffffu, odd ? col[i] : col[i + 2], 1);
              const float g1 = __shfl_xor_sync(0xffffffffu, odd ? col[i + 1] : col[i + 3], 1);
              const int b = h * 64 + c0 + i + (odd ? 2 : 0);
              const uint64_t idx = tbase + dep(eb[b]) + ot;
              if (QSV_IN_BOUNDS(idx + 1, lim))
                __stcs(reinterpret_cast<float4*>(psi + idx),
                       odd ? make_float4(g0, col[i + 2], g1, col[i + 3]) : make_float4(col[i], g0, col[i + 1], g1));
            }
          } else {
  #pragma unroll
            for (int i = 0; i < 32; i += 2) {
              const float got = __shfl_xor_sync(0xffffffffu, odd ? col[i] : col[i + 1], 1);
              const int b = h * 64 + c0 + i + (odd ? 1 : 0);
              const uint64_t idx = tbase + dep(eb[b]) + ot;
              if (QSV_IN_BOUNDS(idx, lim))
                __stcs(psi + idx, odd ? make_float2(got, col[i + 1]) : make_float2(col[i], got));
            }
          }
        }
      } else {
        const int q = warp & 3;
        const int h = warp >> 2;
        const int b = q * 32 + lane;
        const int eb_ = eb[b];
        const uint32_t lane_addr = acc + ((uint32_t)(q * 32) << 16);
        constexpr int CH = P::COLS_PER_WARP < 32 ? P::COLS_PER_WARP : 32;
  #pragma unroll
        for (int c0 = 0; c0 < P::COLS_PER_WARP; c0 += CH) {
          float re[CH], im[CH];
          const int t0 = h * P::COLS_PER_WARP + c0;
          tmem_ld<CH>(lane_addr + (uint32_t)t0, re);
          tmem_ld<CH>(lane_addr + (uint32_t)(P::T + t0), im);
          tmem_ld_wait();
          if constexpr (STAGED) {
  #pragma unroll
            for (int j = 0; j < CH; ++j) raw[slot(eb_ | et[t0 + j])] = make_float2(re[j], im[j]);
          } else if (a.vec == 4 && CH % 4 == 0) {
            const uint64_t rb = tbase + dep(eb_);
  #pragma unroll
            for (int j = 0; j < CH; j += 4)
              if (QSV_IN_BOUNDS(rb + dep(et[t0 + j]) + 3, lim)) st_v8(psi + rb + dep(et[t0 + j]), &re[j], &im[j]);
          } else if (a.vec >= 2) {
            const uint64_t rb = tbase + dep(eb_);
  #pragma unroll
            for (int j = 0; j < CH; j += 2)
              if (QSV_IN_BOUNDS(rb + dep(et[t0 + j]) + 1, lim))
                __stcs(reinterpret_cast<float4*>(psi + rb + dep(et[t0 + j])),
                       make_float4(re[j], im[j], re[j + 1], im[j + 1]));
          } else {
            const uint64_t rb = tbase + dep(eb_);
  #pragma unroll
            for (int j = 0; j < CH; ++j)
              if (QSV_IN_BOUNDS(rb + dep(et[t0 + j]), lim)) __stcs(&psi[rb + dep(et[t0 + j])], make_float2(re[j], im[j]));
          }
        }
      }
  };
  auto operand_ready = [&]() {
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
  };

  uint32_t ph[2] = {0u, 0u};
  bool pending[2] = {false, false};
  // Wait for the products in accumulator s (bounded by a.wait_ns).  With the injected
  // stall, the CTA's first such wait is on stall_bar, which nothing arrives on: it gives
  // up after a.wait_ns and takes the abort path (drain, free TMEM, status word).  Every
  // CTA's first wait comes before its first store, so an aborted launch leaves the state
  // as it was.
  bool stall = a.stall_first != 0;
  auto wait_products = [&](int s) -> bool {
    if (stall) {
      stall = false;
      if (!mbar_wait_bounded(smem_u32(stall_bar), 0u, a.wait_ns)) return false;
    }
    return mbar_wait_bounded(bar_of(s), ph[s], a.wait_ns);
  };
  uint64_t tile = blockIdx.x;
  uint64_t base = 0;
  // Amplitude offset of a tile: its state's start plus the tile's zero-inserted index.
  auto tile_base = [&](uint64_t t) -> uint64_t {
    if (!a.set_tiles) return qsv_insert_zeros(a.reverse ? a.ntiles - 1 - t : t, a.ptile, P::EBITS);
    const uint64_t st = t >> set_shift;
    return st * a.set_amps + qsv_insert_zeros(t - (st << set_shift), a.ptile, P::EBITS);
  };
  // Batches: before a tile of another state is written into the operand, its state's W
  // replaces the current one (callers have no products in flight at that point; the
  // operand_ready() that follows publishes W to the tensor cores).
  auto switch_set = [&](uint64_t t) {
    if (!a.set_tiles) return;
    const uint64_t st = t >> set_shift;
    if (st == cur_set) return;
    cur_set = st;
    load_w(st);
  };
  if (tile < a.ntiles) {
    base = tile_base(tile);
    load_tile(base);
  }
  if constexpr (!SHUF) {
    for (; tile < a.ntiles; tile += gridDim.x) {
      switch_set(tile);
      write_a();
      operand_ready();
      issue_mma(tmem, bar_of(0));
      pending[0] = true;
      // Prefetch the next tile while the tensor cores work.
      const uint64_t next = tile + gridDim.x;
      uint64_t next_base = 0;
      if (next < a.ntiles) {
        next_base = tile_base(next);
        load_tile(next_base);
      }
      if (wait_products(0)) {
        ph[0] ^= 1u;
        pending[0] = false;
      } else {
        atomicExch(abort_flag, 1);
      }
      tc_fence_after();
      __syncthreads();
      if (*abort_flag) break;
      epilogue(base, tmem);
      tc_fence_before();
      __syncthreads();
      if constexpr (STAGED) {
        // Write the tile back in address order.
#pragma unroll
        for (int u = 0; u < P::VEC; ++u) {
          const int e = 2 * (u * FB_THREADS + tid);
          if (QSV_IN_BOUNDS(base + dep(e) + 1, lim)) __stcs(reinterpret_cast<float4*>(psi + base + dep(e)), raw4[slot(e) >> 1]);
        }
        __syncthreads();
      }
      tc_fence_after();
      base = next_base;
    }
  } else {
    uint64_t prev_base = 0;
    int it = 0;
    for (; tile < a.ntiles; tile += gridDim.x, ++it) {
      const int s = it & 1;
      if (it > 0) {
        // Products of the previous tile: A is free again and accumulator s^1 is ready.
        if (wait_products(s ^ 1)) {
          ph[s ^ 1] ^= 1u;
          pending[s ^ 1] = false;
        } else {
          atomicExch(abort_flag, 1);
        }
        tc_fence_after();
      }
      __syncthreads();
      if (*abort_flag) break;
      switch_set(tile);
      write_a();
      operand_ready();
      issue_mma(tmem + (uint32_t)(s * P::KD), bar_of(s));
      pending[s] = true;
      const uint64_t next = tile + gridDim.x;
      uint64_t next_base = 0;
      if (next < a.ntiles) {
        next_base = tile_base(next);
        load_tile(next_base);
      }
      if (it > 0) epilogue(prev_base, tmem + (uint32_t)((s ^ 1) * P::KD));
      tc_fence_before();
      prev_base = base;
      base = next_base;
    }
    if (it > 0 && !*abort_flag) {
      const int s = (it - 1) & 1;
      if (wait_products(s)) {
        ph[s] ^= 1u;
        pending[s] = false;
      } else {
        atomicExch(abort_flag, 1);
      }
      tc_fence_after();
      __syncthreads();
      if (!*abort_flag) epilogue(prev_base, tmem + (uint32_t)(s * P::KD));
    }
  }
  __syncthreads();
  if (*abort_flag) {
    // Products still in flight get a last bounded wait before TMEM is freed.
    for (int s = 0; s < 2; ++s)
      if (pending[s]) mbar_wait_bounded(bar_of(s), ph[s]);
    if (tid == 0) atomicExch(a.flag, 1);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)TCOLS)
                 : "memory");
  }
}

// ---- the tensor-core adjoint's fused backward pass --------------------------------------
// One launch per block over all parameter sets, for blocks in the direct, prefix and pair
// geometries.  Per tile (128 groups x 64 targets of
// one set) it loads psi and lambda, writes both bf16 operand images and issues three
// product sets on the tensor cores: psi U^+ and lambda U^+ (the un-compute, written back
// in place) and the correlation D[m][n] = sum_g psi[g][m] lambda[g][n] over the tile's 128
// groups, with both images read MN-major (the same bytes: a K-major image of rows g is
// an MN-major operand with K = g; core matrices 128 bytes apart along K, 2048 along MN).
// The correlation's running sums stay in TMEM (columns 384..511) and are flushed with
// FP64 atomics into corr[set][m][n] when a CTA leaves a set; the CTAs form 8 groups that
// stride through their sets together (as k_adj_corr_d).  512 threads: two (b, 8 targets)
// items per thread and state, both states of the next tile loaded while the products run.
// psi and lambda are read once and written once per block instead of read twice and
// written once (correlation kernel + two block launches).
struct AdjBackArgs {
  float2* psi;
  float2* lam;
  double* corr;        // [nsets][128][128], accumulated into
  const uint8_t* wimg;  // U^+ image of set s at wimg + s * img_stride
  uint64_t img_stride;
  uint64_t set_amps;    // 2^n
  uint64_t nsets;
  int* flag;
};

constexpr int AB_THREADS = 512;
constexpr int AB_GROUPS = 8;
// psi and lambda images (hi, lo), W (hi, lo), eb, et, dephi, then the mbarrier, the TMEM
// slot and the abort flag.
constexpr int AB_SMEM = 4 * FB<6>::A_BYTES + 2 * FB<6>::W_BYTES + FB_M * 2 + 64 * 2 + 64 * 8 + 64;

// MODE: the block's access mode (direct, prefix, pair1, pair2; the last three multiply
// transposed and take interleaved W images, as in k_block_tc).  Loads in the transposed
// modes: 4 runs of 32 bytes per thread and state with the k_block_tc mappings spread over
// 16 warps (prefix: group ((w%8)*8 + lane/4) | (w/8)*64, targets 4*((lane%4) + 4u) ..;
// pair1: the k_block_tc pair1 roles with group bit 6 on warp bit 3; pair2: target bit 5 on
// warp bit 3), exchanged as there.
template <int MODE>
__global__ void __launch_bounds__(AB_THREADS, 1)
    k_adj_back(const __grid_constant__ BlockArgs g, const __grid_constant__ AdjBackArgs a) {
  using P = FB<6>;
  constexpr bool TRANS = MODE != MODE_DIRECT;
  constexpr int PAIR = MODE == MODE_PAIR1 ? 1 : (MODE == MODE_PAIR2 ? 2 : 0);
  constexpr int ITEMS = (FB_M * (P::T / 8)) / AB_THREADS;  // 2 (direct: (b, 8 targets) items)
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sP_hi = smem;
  uint8_t* sP_lo = smem + P::A_BYTES;
  uint8_t* sL_hi = smem + 2 * P::A_BYTES;
  uint8_t* sL_lo = smem + 3 * P::A_BYTES;
  uint8_t* sW_hi = smem + 4 * P::A_BYTES;
  uint8_t* sW_lo = sW_hi + P::W_BYTES;
  uint16_t* eb = reinterpret_cast<uint16_t*>(sW_lo + P::W_BYTES);
  uint16_t* et = eb + FB_M;
  uint64_t* dephi = reinterpret_cast<uint64_t*>(et + P::T);
  uint64_t* mbar = dephi + P::T;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 1);
  int* abort_flag = reinterpret_cast<int*>(tslot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int i = tid; i < FB_M; i += AB_THREADS) eb[i] = g.eb[i];
  for (int i = tid; i < P::T; i += AB_THREADS) {
    et[i] = g.et[i];
    dephi[i] = g.dephi[i];
  }
  if (tid == 0) {
    mbar_init(smem_u32(mbar), 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(512u)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t accP = tmem, accL = tmem + 128, accC = tmem + 256, sums = tmem + 384;
  auto dep = [&](int e) -> uint64_t { return (uint64_t)(e & (FB_M - 1)) + dephi[e >> FB_BATCH_BITS]; };

  // This CTA's tiles: group grp of the CTAs takes sets grp, grp + ngr, ...; within a set
  // its CTAs stride through the tiles together.
  const uint64_t tps = g.ntiles;  // tiles per set
  uint64_t ngr64 = a.nsets < (uint64_t)gridDim.x ? a.nsets : (uint64_t)gridDim.x;
  if (ngr64 > (uint64_t)AB_GROUPS) ngr64 = AB_GROUPS;
  const int ngr = (int)ngr64;
  const int grp = blockIdx.x % ngr;
  const uint64_t rank = blockIdx.x / ngr;
  const uint64_t nctas = (gridDim.x - grp + ngr - 1) / ngr;
  const uint64_t cnt = rank < tps ? (tps - rank + nctas - 1) / nctas : 0;
  const uint64_t nsg = (a.nsets - grp + ngr - 1) / ngr;
  const uint64_t total = cnt * nsg;
  struct Pos {
    uint64_t set, local, li;
  };
  auto advance = [&](Pos& p) {
    p.local += nctas;
    if (++p.li == cnt) {
      p.li = 0;
      p.local = rank;
      p.set += ngr;
    }
  };
  auto tile_base = [&](const Pos& p) -> uint64_t {
    return p.set * a.set_amps + qsv_insert_zeros(p.local, g.ptile, P::EBITS);
  };
  [[maybe_unused]] const uint64_t lim = a.set_amps * a.nsets;
  // Transposed modes: load u's first group / target and the run held after the exchange.
  auto lb = [&](int i) -> int { return (lane >> i) & 1; };
  auto ld_b = [&](int u) -> int {
    return PAIR == 0 ? (((warp & 7) << 3) | (lane >> 2) | ((warp >> 3) << 6))
           : PAIR == 1 ? (lb(3) << 1) | (lb(4) << 2) | ((warp & 7) << 3) | ((warp >> 3) << 6)
                       : (lb(3) << 2) | (lb(4) << 3) | ((warp & 7) << 4);
  };
  auto ld_t = [&](int u) -> int {
    return PAIR == 0 ? 4 * ((lane & 3) | (u << 2))
           : PAIR == 1 ? (lb(0) << 1) | (lb(1) << 2) | (lb(2) << 3) | (u << 4)
                       : lb(0) | (lb(1) << 1) | (lb(2) << 2) | (u << 3) | ((warp >> 3) << 5);
  };
  auto held_b = [&](int u) -> int {
    return PAIR == 0 ? ld_b(u)
           : PAIR == 1 ? lb(0) | (lb(3) << 1) | (lb(4) << 2) | ((warp & 7) << 3) | ((warp >> 3) << 6)
                       : lb(0) | (lb(1) << 1) | (lb(3) << 2) | (lb(4) << 3) | ((warp & 7) << 4);
  };
  auto held_q4 = [&](int u) -> int {
    return PAIR == 0 ? (lane & 3) | (u << 2) : PAIR == 1 ? lb(1) | (lb(2) << 1) | (u << 2) : lb(2) | (u << 1) | ((warp >> 3) << 3);
  };
  float2 bp[16], bl[16];  // direct: item it, target j at [8*it + j]; transposed: run u, j at [4*u + j]
  auto load = [&](uint64_t base) {
    if constexpr (TRANS) {
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const uint64_t idx = base + dep(eb[ld_b(u)]) + dep(et[ld_t(u)]);
        if (QSV_IN_BOUNDS(idx + 3, lim)) {
          ld_v8(a.psi + idx, &bp[4 * u]);
          ld_v8(a.lam + idx, &bl[4 * u]);
        }
      }
    } else {
#pragma unroll
      for (int it = 0; it < ITEMS; ++it) {
        const int item = it * AB_THREADS + tid;
        const uint64_t rb = base + dep(eb[item & (FB_M - 1)]);
        const int tg = item >> FB_BATCH_BITS;
        if (g.vec == 4) {  // targets t..t+3 adjacent: 32-byte loads
#pragma unroll
          for (int j = 0; j < 8; j += 4) {
            const uint64_t idx = rb + dep(et[tg * 8 + j]);
            if (QSV_IN_BOUNDS(idx + 3, lim)) {
              ld_v8(a.psi + idx, &bp[8 * it + j]);
              ld_v8(a.lam + idx, &bl[8 * it + j]);
            }
          }
        } else if (g.vec == 2) {  // t, t+1 adjacent: 16-byte loads
#pragma unroll
          for (int j = 0; j < 8; j += 2) {
            const uint64_t idx = rb + dep(et[tg * 8 + j]);
            if (!QSV_IN_BOUNDS(idx + 1, lim)) continue;
            const float4 vp = __ldcs(reinterpret_cast<const float4*>(a.psi + idx));
            const float4 vl = __ldcs(reinterpret_cast<const float4*>(a.lam + idx));
            bp[8 * it + j] = make_float2(vp.x, vp.y);
            bp[8 * it + j + 1] = make_float2(vp.z, vp.w);
            bl[8 * it + j] = make_float2(vl.x, vl.y);
            bl[8 * it + j + 1] = make_float2(vl.z, vl.w);
          }
        } else {
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const uint64_t idx = rb + dep(et[tg * 8 + j]);
            if (QSV_IN_BOUNDS(idx, lim)) {
              bp[8 * it + j] = __ldcs(a.psi + idx);
              bl[8 * it + j] = __ldcs(a.lam + idx);
            }
          }
        }
      }
    }
  };
  // Pair modes: turn the loaded runs into runs of 4 targets of one group (as k_block_tc).
  auto exchange = [&](float2* r) {
    if constexpr (PAIR == 1) {
      const bool up = lane & 1;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        float2* x = r + 4 * u;
        const float2 y = x[1];
        x[1] = x[2];
        x[2] = y;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          const float2 send = up ? x[j] : x[j + 2];
          float2 got;
          got.x = __shfl_xor_sync(0xffffffffu, send.x, 1);
          got.y = __shfl_xor_sync(0xffffffffu, send.y, 1);
          if (up)
            x[j] = got;
          else
            x[j + 2] = got;
        }
      }
    } else if constexpr (PAIR == 2) {
#pragma unroll
      for (int bb = 0; bb < 2; ++bb) {
        const bool up = (lane >> bb) & 1;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          float2* x = r + 4 * u;
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            if (j & (1 << bb)) continue;
            const int j1 = j | (1 << bb);
            const float2 send = up ? x[j] : x[j1];
            float2 got;
            got.x = __shfl_xor_sync(0xffffffffu, send.x, 1 << bb);
            got.y = __shfl_xor_sync(0xffffffffu, send.y, 1 << bb);
            if (up)
              x[j] = got;
            else
              x[j1] = got;
          }
        }
      }
    }
  };
  auto write_image = [&](const float2* buf, uint8_t* hi, uint8_t* lo) {
    if constexpr (TRANS) {
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int b = held_b(u), q4 = held_q4(u);
        float re[4], im[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          re[j] = buf[4 * u + j].x;
          im[j] = buf[4 * u + j].y;
        }
        uint2 rh, rl, ih, il;
        split4(re, rh, rl);
        split4(im, ih, il);
        const int off_re = (q4 >> 1) * P::A_LBO + b * 16 + (q4 & 1) * 8;
        const int off_im = off_re + (P::T / 8) * P::A_LBO;
        *reinterpret_cast<uint2*>(hi + off_re) = rh;
        *reinterpret_cast<uint2*>(lo + off_re) = rl;
        *reinterpret_cast<uint2*>(hi + off_im) = ih;
        *reinterpret_cast<uint2*>(lo + off_im) = il;
      }
    } else {
#pragma unroll
      for (int it = 0; it < ITEMS; ++it) {
        const int item = it * AB_THREADS + tid;
        const int b = item & (FB_M - 1);
        const int tg = item >> FB_BATCH_BITS;
        float re[8], im[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          re[j] = buf[8 * it + j].x;
          im[j] = buf[8 * it + j].y;
        }
        uint4 rh, rl, ih, il;
        split8(re, rh, rl);
        split8(im, ih, il);
        const int off_re = tg * P::A_LBO + b * 16;
        const int off_im = (P::T / 8 + tg) * P::A_LBO + b * 16;
        *reinterpret_cast<uint4*>(hi + off_re) = rh;
        *reinterpret_cast<uint4*>(lo + off_re) = rl;
        *reinterpret_cast<uint4*>(hi + off_im) = ih;
        *reinterpret_cast<uint4*>(lo + off_im) = il;
      }
    }
  };
  uint64_t cur_set = ~0ull;
  auto load_w = [&](uint64_t set) {
    const uint4* src = reinterpret_cast<const uint4*>(a.wimg + set * a.img_stride);
    uint4* dst = reinterpret_cast<uint4*>(sW_hi);
    constexpr int NV = (2 * P::W_BYTES) / 16;
    for (int i = tid; i < NV; i += AB_THREADS) dst[i] = src[i];
  };
  constexpr uint32_t idesc = make_idesc(FB_M, P::KD);
  // Correlation: both operands MN-major (transpose bits 15, 16), K = the tile's groups.
  constexpr uint32_t idesc_c = make_idesc(P::KD, P::KD) | (1u << 15) | (1u << 16);
  auto issue = [&]() {
    if (tid != 0) return;
    const uint32_t ph = smem_u32(sP_hi), pl = smem_u32(sP_lo), lh = smem_u32(sL_hi), ll = smem_u32(sL_lo);
    const uint32_t wh = smem_u32(sW_hi), wl = smem_u32(sW_lo);
    constexpr int KS = P::KD / 16;  // 8 steps of 16 components (block products)
    auto blk = [&](uint32_t acc, uint32_t xh, uint32_t xl) {
      auto mma = [&](uint32_t x, uint32_t w, int s, uint32_t accumulate) {
        const uint64_t td = make_smem_desc(x + s * 2 * P::A_LBO, P::A_LBO, 128);
        const uint64_t wd = make_smem_desc(w + s * 2 * P::W_LBO, P::W_LBO, 128);
        if constexpr (TRANS)
          tc_mma(acc, wd, td, idesc, accumulate);
        else
          tc_mma(acc, td, wd, idesc, accumulate);
      };
      // Corrections first, main pass last (as in k_block_tc).
#pragma unroll
      for (int s = 0; s < KS; ++s) mma(xh, wl, s, s > 0 ? 1u : 0u);
#pragma unroll
      for (int s = 0; s < KS; ++s) mma(xl, wh, s, 1u);
#pragma unroll
      for (int s = 0; s < KS; ++s) mma(xh, wh, s, 1u);
    };
    blk(accP, ph, pl);
    blk(accL, lh, ll);
    constexpr int GS = FB_M / 16;  // 8 steps of 16 groups (correlation)
    auto mn = [&](uint32_t base, int s) { return make_smem_desc(base + s * 256, 128, P::A_LBO); };
#pragma unroll
    for (int s = 0; s < GS; ++s) tc_mma(accC, mn(ph, s), mn(ll, s), idesc_c, s > 0 ? 1u : 0u);
#pragma unroll
    for (int s = 0; s < GS; ++s) tc_mma(accC, mn(pl, s), mn(lh, s), idesc_c, 1u);
#pragma unroll
    for (int s = 0; s < GS; ++s) tc_mma(accC, mn(ph, s), mn(lh, s), idesc_c, 1u);
    tc_commit(smem_u32(mbar));
  };
  const int q = warp & 3, h = warp >> 2;
  const uint32_t lane_off = (uint32_t)(q * 32) << 16;
  // Epilogue of a block product.  Direct: warp w reads TMEM lanes 32*(w%4).. (groups) and
  // target columns [16*(w/4), +16).  Transposed: lane row 32q + lane is component lane%2
  // of target (32q + lane)/2 and warp quarter h reads groups [32h, 32h + 32); lane pairs
  // swap halves so the even lane keeps group b and the odd lane group b+1.
  auto store = [&](uint32_t acc, float2* dst, uint64_t base) {
    if constexpr (TRANS) {
      const bool odd = lane & 1;
      const uint64_t ot = dep(et[(q * 32 + lane) >> 1]);
      float col[32];
      tmem_ld<32>(acc + lane_off + (uint32_t)(h * 32), col);
      tmem_ld_wait();
      if constexpr (PAIR == 2) {  // 16-byte stores of groups b, b+1 (even) / b+2, b+3 (odd)
#pragma unroll
        for (int i = 0; i < 32; i += 4) {
          const float g0 = __shfl_xor_sync(0xffffffffu, odd ? col[i] : col[i + 2], 1);
          const float g1 = __shfl_xor_sync(0xffffffffu, odd ? col[i + 1] : col[i + 3], 1);
          const int b = h * 32 + i + (odd ? 2 : 0);
          const uint64_t idx = base + dep(eb[b]) + ot;
          if (QSV_IN_BOUNDS(idx + 1, lim))
            __stcs(reinterpret_cast<float4*>(dst + idx),
                   odd ? make_float4(g0, col[i + 2], g1, col[i + 3]) : make_float4(col[i], g0, col[i + 1], g1));
        }
      } else {
#pragma unroll
        for (int i = 0; i < 32; i += 2) {
          const float got = __shfl_xor_sync(0xffffffffu, odd ? col[i] : col[i + 1], 1);
          const int b = h * 32 + i + (odd ? 1 : 0);
          const uint64_t idx = base + dep(eb[b]) + ot;
          if (QSV_IN_BOUNDS(idx, lim)) __stcs(dst + idx, odd ? make_float2(got, col[i + 1]) : make_float2(col[i], got));
        }
      }
    } else {
      const int b = q * 32 + lane;
      const uint64_t rb = base + dep(eb[b]);
      const int t0 = h * 16;
      float re[16], im[16];
      tmem_ld<16>(acc + lane_off + (uint32_t)t0, re);
      tmem_ld<16>(acc + lane_off + (uint32_t)(P::T + t0), im);
      tmem_ld_wait();
      if (g.vec == 4) {
#pragma unroll
        for (int j = 0; j < 16; j += 4) {
          const uint64_t idx = rb + dep(et[t0 + j]);
          if (QSV_IN_BOUNDS(idx + 3, lim)) st_v8(dst + idx, &re[j], &im[j]);
        }
      } else if (g.vec == 2) {
#pragma unroll
        for (int j = 0; j < 16; j += 2) {
          const uint64_t idx = rb + dep(et[t0 + j]);
          if (QSV_IN_BOUNDS(idx + 1, lim))
            __stcs(reinterpret_cast<float4*>(dst + idx), make_float4(re[j], im[j], re[j + 1], im[j + 1]));
        }
      } else {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const uint64_t idx = rb + dep(et[t0 + j]);
          if (QSV_IN_BOUNDS(idx, lim)) __stcs(dst + idx, make_float2(re[j], im[j]));
        }
      }
    }
  };
  // Correlation: thread (lane row 32q + lane, columns 32h ..) adds its 32 entries.
  const uint32_t c_off = lane_off + (uint32_t)(h * 32);
  auto zero_sums = [&]() {
    float z[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) z[k] = 0.f;
    tmem_st16(sums + c_off, z);
    tmem_st16(sums + c_off + 16, z);
    tmem_st_wait();
  };
  auto add_corr = [&]() {
#pragma unroll
    for (int c = 0; c < 32; c += 16) {
      float d[16], sv[16];
      tmem_ld<16>(accC + c_off + (uint32_t)c, d);
      tmem_ld<16>(sums + c_off + (uint32_t)c, sv);
      tmem_ld_wait();
#pragma unroll
      for (int k = 0; k < 16; ++k) sv[k] += d[k];
      tmem_st16(sums + c_off + (uint32_t)c, sv);
    }
    tmem_st_wait();
  };
  auto flush = [&](uint64_t set) {
    double* dst = a.corr + set * (uint64_t)(P::KD * P::KD) + (uint64_t)(q * 32 + lane) * P::KD + h * 32;
#pragma unroll
    for (int c = 0; c < 32; c += 16) {
      float sv[16];
      tmem_ld<16>(sums + c_off + (uint32_t)c, sv);
      tmem_ld_wait();
#pragma unroll
      for (int k = 0; k < 16; ++k)
        if (sv[k] != 0.f) atomicAdd(dst + c + k, (double)sv[k]);
    }
    zero_sums();
  };

  zero_sums();
  uint32_t phase = 0;
  bool pending = false;
  Pos cu{(uint64_t)grp, rank, 0}, pf = cu;
  uint64_t base = 0;
  if (total > 0) {
    base = tile_base(pf);
    load(base);
  }
  advance(pf);
  for (uint64_t i = 0; i < total; ++i) {
    if (cu.set != cur_set) {  // no products in flight here
      cur_set = cu.set;
      load_w(cur_set);
    }
    exchange(bp);
    exchange(bl);
    write_image(bp, sP_hi, sP_lo);
    write_image(bl, sL_hi, sL_lo);
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    issue();
    pending = true;
    uint64_t next_base = 0;
    if (i + 1 < total) {
      next_base = tile_base(pf);
      load(next_base);
    }
    advance(pf);
    if (warp == 0) {
      const bool done = mbar_wait_bounded(smem_u32(mbar), phase);
      if (!done && lane == 0) atomicExch(abort_flag, 1);
    }
    phase ^= 1u;
    pending = false;
    __syncthreads();
    tc_fence_after();
    if (*abort_flag) {
      pending = true;
      phase ^= 1u;
      break;
    }
    store(accP, a.psi, base);
    store(accL, a.lam, base);
    add_corr();
    tc_fence_before();
    const uint64_t set = cu.set;
    advance(cu);
    if (cu.li == 0) flush(set);
    base = next_base;
  }
  __syncthreads();
  if (*abort_flag) {
    if (pending) mbar_wait_bounded(smem_u32(mbar), phase);
    if (tid == 0) atomicExch(a.flag, 3);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512u) : "memory");
  }
}

// ---- host: W images ---------------------------------------------------------------------
// The transposed modes (prefix, pair) take W with interleaved rows.
bool uses_interleaved_image(int mode) { return mode == MODE_PREFIX || mode == MODE_PAIR1 || mode == MODE_PAIR2; }

uint16_t f32_to_bf16_rn(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return (uint16_t)((u >> 16) | ((u & 0xffffu) ? 0x40u : 0u));
  const uint32_t rounding = 0x7fffu + ((u >> 16) & 1u);
  return (uint16_t)((u + rounding) >> 16);
}
float bf16_to_f32(uint16_t h) {
  const uint32_t u = (uint32_t)h << 16;
  float f;
  memcpy(&f, &u, 4);
  return f;
}

size_t image_bytes(int k) {
  const size_t kd = size_t(2) << k;
  return 2 * kd * kd * 2;  // hi + lo
}

// Builds the hi/lo bf16 images of W = [[Ur, -Ui], [Ui, Ur]] in the K-major canonical
// layout: element (row nn, col kk) at (kk/8)*(KD*16) + nn*16 + (kk%8)*2.  Rows and
// columns follow the kernel target order: U is read at (tperm[t'], tperm[t]).  With
// interleaved rows (the prefix mode) row nn is component nn & 1 of output t' = nn >> 1.
void build_image(int k, const double* U, const uint8_t* tperm, uint8_t* out, bool interleaved = false) {
  const int T = 1 << k, KD = 2 * T;
  uint16_t* hi = reinterpret_cast<uint16_t*>(out);
  uint16_t* lo = reinterpret_cast<uint16_t*>(out + (size_t)KD * KD * 2);
  for (int nn = 0; nn < KD; ++nn) {
    const int tp = tperm[interleaved ? nn >> 1 : nn % T];
    const bool out_im = interleaved ? (nn & 1) != 0 : nn >= T;
    for (int kk = 0; kk < KD; ++kk) {
      const int t = tperm[kk % T];
      const bool in_im = kk >= T;
      const double ur = U[2 * ((size_t)tp * T + t)], ui = U[2 * ((size_t)tp * T + t) + 1];
      double w;
      if (!out_im)
        w = in_im ? -ui : ur;
      else
        w = in_im ? ur : ui;
      const float wf = (float)w;
      const uint16_t h = f32_to_bf16_rn(wf);
      const uint16_t l = f32_to_bf16_rn((float)(w - (double)bf16_to_f32(h)));
      const size_t e = ((size_t)(kk / 8) * (KD * 16) + (size_t)nn * 16 + (size_t)(kk % 8) * 2) / 2;
      hi[e] = h;
      lo[e] = l;
    }
  }
}

// Shuffle-mode tables (see BlockArgs).  Element e of the tile is named by its bit
// roles: lane bits 0..4 (address bits 0..4), warp bits and register bits.  Returns false
// (the caller then stages the tile) if a table would not cover every tile bit once.
bool shuffle_tables(int k, const int* tpos, const int* batch, const int* eidx, int j, BlockArgs& a) {
  const int T = 1 << k, R = T / 2, ebits = FB_BATCH_BITS + k;
  constexpr int A_LBO = FB_M * 16;
  int kt[8];  // kernel target order: positions ascending
  for (int i = 0; i < k; ++i) kt[i] = tpos[i];
  std::sort(kt, kt + k);
  int tE[8];       // e of kernel target bit i
  int tbit[24];    // kernel target bit of e, or -1
  bool isb[24];    // e is a group (batch) bit
  for (int e = 0; e < ebits; ++e) {
    tbit[e] = -1;
    isb[e] = false;
  }
  for (int i = 0; i < k; ++i) {
    tE[i] = eidx[kt[i]];
    tbit[tE[i]] = i;
  }
  for (int i = 0; i < FB_BATCH_BITS; ++i) isb[eidx[batch[i]]] = true;
  for (int tp = 0; tp < T; ++tp) {
    int t = 0;
    for (int i = 0; i < k; ++i) {
      if (!((tp >> i) & 1)) continue;
      int jj = 0;
      while (tpos[jj] != kt[i]) ++jj;
      t |= 1 << (k - 1 - jj);
    }
    a.tperm[tp] = (uint8_t)t;
  }
  if (j < 1 || j > k - 1) return false;
  const int s = std::min(j, 3);
  // Register bits before the load rounds: group bits above address bit 4 in 0..s-1
  // (they trade places with the first s lane targets), t' bits s..2, then the rest.
  int hb[16], nhb = 0;
  for (int e = 5; e < ebits; ++e)
    if (isb[e]) hb[nhb++] = e;
  int reg[8], wb[3];
  bool used[24] = {false};
  for (int i = 0; i < 3; ++i) {
    reg[i] = i < s ? hb[i] : tE[i];
    used[reg[i]] = true;
  }
  int rest[24], nr = 0;
  for (int e = 5; e < ebits; ++e)
    if (!used[e]) rest[nr++] = e;
  if (nr != k - 1) return false;
  for (int i = 3; i < k - 1; ++i) reg[i] = rest[i - 3];
  for (int i = 0; i < 3; ++i) wb[i] = rest[k - 4 + i];
  a.nld = s;
  for (int i = 0; i < 3; ++i) a.ld_lane[i] = i < s ? tE[i] : 0;
  for (int i = 0; i < 3; ++i) a.ld_warp[i] = 1ull << a.ptile[wb[i]];
  for (int r = 0; r < 32; ++r) {
    uint64_t off = 0;
    for (int i = 0; i < k - 1; ++i)
      if (r < R && ((r >> i) & 1)) off += 1ull << a.ptile[reg[i]];
    a.ld_reg[r] = off;
  }
  int lane_after[5], reg_after[8];
  for (int x = 0; x < 5; ++x) lane_after[x] = x;
  for (int i = 0; i < k - 1; ++i) reg_after[i] = reg[i];
  for (int i = 0; i < s; ++i) {
    lane_after[tE[i]] = reg[i];
    reg_after[i] = tE[i];
  }
  // A row order m: row bits 0..2 = the group bits on lane bits 0..2 (distinct 16-byte
  // slots per quarter warp), then the remaining group bits below address bit 5, then the rest.
  int mb[FB_BATCH_BITS], nm = 0, mbit[24];
  bool placed[24] = {false};
  for (int x = 0; x < 3; ++x) {
    if (!isb[lane_after[x]]) return false;
    mb[nm++] = lane_after[x];
    placed[lane_after[x]] = true;
  }
  for (int e = 0; e < 5; ++e)
    if (isb[e] && !placed[e]) {
      mb[nm++] = e;
      placed[e] = true;
    }
  for (int e = 5; e < ebits && nm < FB_BATCH_BITS; ++e)
    if (isb[e] && !placed[e]) {
      mb[nm++] = e;
      placed[e] = true;
    }
  if (nm != FB_BATCH_BITS) return false;
  for (int i = 0; i < FB_BATCH_BITS; ++i) mbit[mb[i]] = i;
  auto contrib_a = [&](int e) -> uint32_t {
    if (isb[e]) return 16u << mbit[e];
    return (uint32_t)A_LBO << (tbit[e] - 3);
  };
  // Load side: lane_after, warp bits and reg_after bits 3.. must cover every bit once,
  // with t' bits 0..2 exactly on register bits 0..2.
  {
    int cover[24] = {0};
    for (int x = 0; x < 5; ++x) cover[lane_after[x]]++;
    for (int i = 0; i < 3; ++i) cover[wb[i]]++;
    for (int i = 0; i < k - 1; ++i) cover[reg_after[i]]++;
    for (int e = 0; e < ebits; ++e)
      if (cover[e] != 1) return false;
    for (int i = 0; i < 3; ++i)
      if (tbit[reg_after[i]] != i) return false;
    for (int x = 0; x < 5; ++x)
      if (!isb[lane_after[x]] && tbit[lane_after[x]] < 3) return false;
    for (int i = 0; i < 3; ++i)
      if (!isb[wb[i]] && tbit[wb[i]] < 3) return false;
    for (int i = 3; i < k - 1; ++i)
      if (!isb[reg_after[i]] && tbit[reg_after[i]] < 3) return false;
  }
  for (int x = 0; x < 5; ++x) a.a_lw[x] = contrib_a(lane_after[x]);
  for (int i = 0; i < 3; ++i) a.a_lw[5 + i] = contrib_a(wb[i]);
  for (int it = 0; it < 4; ++it) {
    uint32_t off = 0;
    for (int y = 0; 3 + y < k - 1; ++y)
      if (it < R / 8 && ((it >> y) & 1)) off += contrib_a(reg_after[3 + y]);
    a.a_it[it] = off;
  }
  // Epilogue: row bits 0..4 on the lanes; the j of them above address bit 4 trade
  // places with register bits 0..j-1 (t' bits 0..j-1, the targets below bit 5).
  int es[5], nes = 0;
  for (int x = 0; x < 5; ++x)
    if (mb[x] >= 5) es[nes++] = x;
  if (nes != j) return false;
  int lane_epi[5], reg_epi[8];
  for (int x = 0; x < 5; ++x) lane_epi[x] = mb[x];
  for (int i = 0; i < k - 1; ++i) reg_epi[i] = tE[i];
  for (int i = 0; i < j; ++i) {
    lane_epi[es[i]] = tE[i];
    reg_epi[i] = mb[es[i]];
  }
  {
    int cover[24] = {0};
    for (int x = 0; x < 5; ++x) {
      if (lane_epi[x] >= 5) return false;
      cover[lane_epi[x]]++;
    }
    cover[mb[5]]++;
    cover[mb[6]]++;
    cover[tE[k - 1]]++;
    for (int i = 0; i < k - 1; ++i) cover[reg_epi[i]]++;
    for (int e = 0; e < ebits; ++e)
      if (cover[e] != 1) return false;
  }
  a.nst = j;
  for (int i = 0; i < 5; ++i) a.st_lane[i] = i < j ? es[i] : 0;
  for (int x = 0; x < 5; ++x) a.st_lw[x] = 1ull << a.ptile[lane_epi[x]];
  a.st_lw[5] = 1ull << a.ptile[mb[5]];
  a.st_lw[6] = 1ull << a.ptile[mb[6]];
  a.st_lw[7] = 1ull << a.ptile[tE[k - 1]];
  for (int c = 0; c < 32; ++c) {
    uint64_t off = 0;
    for (int i = 0; i < k - 1; ++i)
      if (c < R && ((c >> i) & 1)) off += 1ull << a.ptile[reg_epi[i]];
    a.st_reg[c] = off;
  }
  return true;
}

// Tile geometry of a block on target positions tpos[0..k) (tpos[0] = MSB of t):
// sorted tile positions, the e-index maps of groups and targets, the address table
// and the staging swizzle (see BlockArgs).
// user_pos is the caller's target order (user_pos[0] = MSB of the block matrix index).
// The kernels see the targets in descending bit order (the block matrix is permuted
// to match through tperm), so an access mode means the same thing for every order of a
// placement.  forced_mode >= 0 replaces the built-in rule where it applies.
void tile_geometry(int k, const int* user_pos, BlockArgs& a, int forced_mode) {
  const int ebits = FB_BATCH_BITS + k;
  int tpos[8];
  for (int j = 0; j < k; ++j) tpos[j] = user_pos[j];
  std::sort(tpos, tpos + k, [](int x, int y) { return x > y; });
  uint64_t tmask = 0;
  for (int j = 0; j < k; ++j) tmask |= 1ull << tpos[j];
  // Lanes of a warp cover address bits 0..4.  With j targets there, direct accesses
  // stay coalesced only when those targets are the address prefix 0..L-1 with L <= 2
  // (L == j; t's lowest bits are exactly those, as tpos is in descending bit order, so
  // t..t+vec-1 are adjacent amplitudes and a warp reads 32 x vec contiguous
  // amplitudes; a longer prefix spreads the lanes 2^L amplitudes apart).  A 6-qubit block
  // with a prefix of 4 or more runs transposed (prefix mode; measured faster there than
  // the direct and shuffle modes, and slower at L = 3).  Otherwise the shuffle mode
  // handles up to k-1 of them and the staged mode the rest.
  int L = 0;
  while (L < k && tpos[k - 1 - L] == L) ++L;
  const int jl = __builtin_popcountll(tmask & 0x1Full);
  a.vec = L >= 2 ? 4 : (L == 1 ? 2 : 1);
  // A 6-qubit block whose lowest target sits on bit 1 (2) takes pair1 (pair2) when at
  // least 3 of bits 1..4 (2..5) are targets: measured faster than shuffle for every such
  // class, and slower with fewer (the store runs break up).
  const bool run1 = k == 6 && tpos[k - 1] == 1 && __builtin_popcountll(tmask & 0x1Eull) >= 3;
  const bool run2 = k == 6 && tpos[k - 1] == 2 && __builtin_popcountll(tmask & 0x3Cull) >= 3;
  // Direct also wins (or ties) for a prefix of 3 and whenever no target sits on address
  // bits 0..2 (measured at n=26 for k = 4, 5, 6: e.g. bits 4..6 0.183 ms against 0.195
  // shuffle, bits 0..2 0.190 against 0.201 prefix and 0.227 shuffle).
  const bool low3_free = tpos[k - 1] >= 3;
  const int rule = (jl == L && L <= 3) ? MODE_DIRECT
                   : (k == 6 && L >= 4) ? MODE_PREFIX
                   : run1               ? MODE_PAIR1
                   : run2               ? MODE_PAIR2
                   : low3_free          ? MODE_DIRECT
                                        : (jl <= k - 1 ? MODE_SHUF : MODE_STAGED);
  a.mode = rule;
  if (forced_mode == MODE_DIRECT || forced_mode == MODE_STAGED) a.mode = forced_mode;
  if (forced_mode == MODE_SHUF && jl >= 1 && jl <= k - 1) a.mode = MODE_SHUF;
  if (forced_mode == MODE_PREFIX && k == 6 && L >= 3) a.mode = MODE_PREFIX;
  // Any placement with the lowest target on bit 1 (pair1) or 2 (pair2) is correct in the
  // pair modes; the run of 4 only decides how whole the store runs are.
  if ((forced_mode == MODE_PAIR1 && k == 6 && tpos[k - 1] == 1) ||
      (forced_mode == MODE_PAIR2 && k == 6 && tpos[k - 1] == 2))
    a.mode = forced_mode;
  int batch[FB_BATCH_BITS];
  for (int p = 0, nb = 0; nb < FB_BATCH_BITS; ++p)
    if (!((tmask >> p) & 1ull)) batch[nb++] = p;
  uint64_t pmask = tmask;
  for (int i = 0; i < FB_BATCH_BITS; ++i) pmask |= 1ull << batch[i];
  int eidx[64];
  for (int p = 0, e = 0; p < 64; ++p)
    if ((pmask >> p) & 1ull) {
      a.ptile[e] = p;
      eidx[p] = e++;
    }
  for (int b = 0; b < FB_M; ++b) {
    int e = 0;
    for (int i = 0; i < FB_BATCH_BITS; ++i)
      if ((b >> i) & 1) e |= 1 << eidx[batch[i]];
    a.eb[b] = (uint16_t)e;
  }
  const int T = 1 << k;
  for (int t = 0; t < T; ++t) {
    int e = 0;
    for (int j = 0; j < k; ++j)
      if ((t >> (k - 1 - j)) & 1) e |= 1 << eidx[tpos[j]];
    a.et[t] = (uint16_t)e;
  }
  for (int x = 0; x < (1 << (ebits - FB_BATCH_BITS)); ++x) {
    uint64_t off = 0;
    for (int j = 0; j < ebits - FB_BATCH_BITS; ++j)
      if ((x >> j) & 1) off |= 1ull << a.ptile[FB_BATCH_BITS + j];
    a.dephi[x] = off;
  }
  // Swizzle: lanes of a warp hold 32 consecutive b, i.e. vary the e-bits of batch bits
  // 0..4.  Word position of e in a 128-byte row = (e & 15) ^ (swz << 1); choose the
  // 3-bit constant of each e-bit >= 4 so those lanes span as many word positions as
  // possible (rank over GF(2)); e-bits < 4 contribute themselves.
  int c[16] = {0};
  unsigned span[16];  // basis vectors (4-bit) by leading bit
  for (int i = 0; i < 16; ++i) span[i] = 0;
  auto insert = [&](unsigned v) -> bool {
    for (int bit = 3; bit >= 0; --bit) {
      if (!((v >> bit) & 1u)) continue;
      if (!span[bit]) {
        span[bit] = v;
        return true;
      }
      v ^= span[bit];
    }
    return false;
  };
  for (int i = 0; i < 5; ++i) {
    const int e = eidx[batch[i]];
    if (e < 4) insert(1u << e);
  }
  for (int i = 0; i < 5; ++i) {
    const int e = eidx[batch[i]];
    if (e < 4) continue;
    for (unsigned cand = 1; cand < 8; ++cand) {
      if (insert(cand << 1)) {
        c[e] = (int)cand;
        break;
      }
    }
  }
  for (int y = 0; y < (1 << (ebits - 4)); ++y) {
    int v = 0;
    for (int jj = 0; jj < ebits - 4; ++jj)
      if ((y >> jj) & 1) v ^= c[4 + jj];
    a.swz[y] = (uint8_t)v;
  }
  if (a.mode == MODE_SHUF && !shuffle_tables(k, user_pos, batch, eidx, jl, a)) a.mode = MODE_STAGED;
  if (a.mode != MODE_SHUF) {
    // Sorted index t (bit k-1-i <-> tpos[i]) -> caller's index (bit k-1-jj <-> user_pos[jj]).
    for (int t = 0; t < T; ++t) {
      int u = 0;
      for (int i = 0; i < k; ++i) {
        if (!((t >> (k - 1 - i)) & 1)) continue;
        int jj = 0;
        while (user_pos[jj] != tpos[i]) ++jj;
        u |= 1 << (k - 1 - jj);
      }
      a.tperm[t] = (uint8_t)u;
    }
  }
}

// ---- measured access modes ---------------------------------------------------------------
// Per device: the access mode to use for a placement class (k, target bits among address
// bits 0..6), set by qsv_tune_blocks (fastest measured) or qsv_set_block_mode.
std::mutex g_mode_mu;
std::map<long long, int> g_modes;

long long mode_key(int dev, int k, int low) { return ((long long)dev << 16) | ((long long)k << 8) | low; }

int lookup_mode(int dev, int k, int low) {
  std::lock_guard<std::mutex> lk(g_mode_mu);
  auto it = g_modes.find(mode_key(dev, k, low));
  return it == g_modes.end() ? -1 : it->second;
}

bool mode_applies(int k, int low, int mode) {
  if (mode == MODE_DIRECT || mode == MODE_STAGED) return true;
  if (mode == MODE_PREFIX) return k == 6 && (low & 7) == 7;  // targets on address bits 0, 1, 2
  if (mode == MODE_PAIR1) return k == 6 && (low & 3) == 2;  // lowest target on bit 1
  if (mode == MODE_PAIR2) return k == 6 && (low & 7) == 4;  // lowest target on bit 2
  const int j = __builtin_popcount((unsigned)low & 0x1Fu);
  return mode == MODE_SHUF && j >= 1 && j <= k - 1;
}

// One launch of the fused-block kernel: one CTA per SM (TMEM and shared memory allow no
// more at k = 6), persistent over the tiles.
template <int KQ, int MODE>
cudaError_t launch_fb(const BlockArgs& a, float2* psi, cudaStream_t stream, int sm_count) {
  using P = FB<KQ>;
  constexpr int SMEM = MODE == MODE_STAGED ? P::SMEM : P::SMEM_DIRECT;
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(k_block_tc<KQ, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  int per_sm = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_block_tc<KQ, MODE>, FB_THREADS, SMEM);
  if (per_sm < 1) per_sm = 1;
  // Bound co-resident CTAs so their TMEM allocations always fit (512 columns per SM).
  per_sm = std::min(per_sm, 512 / (MODE == MODE_SHUF ? P::TMEM_COLS2 : P::TMEM_COLS));
  uint64_t grid = (uint64_t)std::max(1, sm_count) * per_sm;
  if (grid > a.ntiles) grid = a.ntiles;
  k_block_tc<KQ, MODE><<<(unsigned)grid, FB_THREADS, SMEM, stream>>>(psi, a);
  return cudaGetLastError();
}

template <int KQ, int MODE>
int launch_block_variant(qsv_state* s, const BlockArgs& args, float2* psi) {
  using P = FB<KQ>;
  BlockArgs a = args;
  a.wait_ns = FB_WAIT_NS;
  a.stall_first = 0;
  if (s->inject_stall_ns) {  // armed by qsv_inject_block_stall for this one launch
    a.wait_ns = s->inject_stall_ns;
    a.stall_first = 1;
    s->inject_stall_ns = 0;
  }
  cudaError_t e = launch_fb<KQ, MODE>(a, psi, s->stream, s->sm_count);
  if (e != cudaSuccess) return set_error(s, QSV_ERR_CUDA, "block_tc launch: %s", cudaGetErrorString(e));
  return check_launch(s, "block_tc");
}

template <int KQ>
int launch_block(qsv_state* s, const BlockArgs& a, float2* psi) {
  switch (a.mode) {
    case MODE_STAGED: return launch_block_variant<KQ, MODE_STAGED>(s, a, psi);
    case MODE_SHUF: return launch_block_variant<KQ, MODE_SHUF>(s, a, psi);
    case MODE_PREFIX:
      if constexpr (KQ == 6) return launch_block_variant<KQ, MODE_PREFIX>(s, a, psi);
      return set_error(s, QSV_ERR_INVALID, "prefix mode on a %d-qubit block", KQ);
    case MODE_PAIR1:
      if constexpr (KQ == 6) return launch_block_variant<KQ, MODE_PAIR1>(s, a, psi);
      return set_error(s, QSV_ERR_INVALID, "pair mode on a %d-qubit block", KQ);
    case MODE_PAIR2:
      if constexpr (KQ == 6) return launch_block_variant<KQ, MODE_PAIR2>(s, a, psi);
      return set_error(s, QSV_ERR_INVALID, "pair mode on a %d-qubit block", KQ);
    default: return launch_block_variant<KQ, MODE_DIRECT>(s, a, psi);
  }
}

}  // namespace

struct qsv_plan {
  int nblocks = 0;
  void* d_images = nullptr;
  std::vector<BlockArgs> args;
  int n = 0;
};

namespace {
int launch_args_on(qsv_state* s, const BlockArgs& a, float2* psi) {
  switch (a.k) {
    case 4: return launch_block<4>(s, a, psi);
    case 5: return launch_block<5>(s, a, psi);
    default: return launch_block<6>(s, a, psi);
  }
}

// Consecutive launches on a state alternate the tile order (serpentine): each starts
// with the tiles the previous one wrote last, part of which is still in L2 (measured
// 0.2-0.5% per step on the brickwork plan; normal-priority stores instead of streaming
// ones, to keep more of them there, measured 3.5% slower).
int launch_args(qsv_state* s, const BlockArgs& args) {
  BlockArgs a = args;
  a.reverse = (int)(s->block_launches++ & 1);
  return launch_args_on(s, a, (float2*)s->d_amp);
}

// Validates a block list and fills per-block launch arguments and image offsets.
int prepare_blocks(qsv_state* s, int nblocks, const int* ks, const int* targets_flat,
                   std::vector<BlockArgs>& args, std::vector<size_t>& img_off,
                   std::vector<size_t>& mat_offs, size_t& total) {
  total = 0;
  size_t mat_off = 0;
  int tofs = 0;
  args.assign((size_t)nblocks, BlockArgs{});
  img_off.assign((size_t)nblocks, 0);
  mat_offs.assign((size_t)nblocks, 0);
  for (int i = 0; i < nblocks; ++i) {
    const int k = ks[i];
    if (k < 4 || k > 6) return set_error(s, QSV_ERR_INVALID, "block %d: k=%d outside [4, 6]", i, k);
    if (s->n - k < FB_BATCH_BITS)
      return set_error(s, QSV_ERR_UNSUPPORTED, "block %d: n=%d too small for a %d-qubit tensor-core block", i,
                       s->n, k);
    BlockArgs& a = args[(size_t)i];
    uint64_t seen = 0;
    int tpos[8];
    int rc = to_positions(s, k, targets_flat + tofs, tpos, &seen);
    if (rc) return rc;
    a.k = k;
    a.ntiles = 1ull << (s->n - k - FB_BATCH_BITS);
    int low = 0;
    for (int j = 0; j < k; ++j)
      if (tpos[j] < FB_BATCH_BITS) low |= 1 << tpos[j];
    tile_geometry(k, tpos, a, lookup_mode(s->device, k, low));
    a.flag = s->d_flag;
    img_off[(size_t)i] = total;
    mat_offs[(size_t)i] = mat_off;
    total += image_bytes(k);
    mat_off += (size_t)2 << (2 * k);
    tofs += k;
  }
  return QSV_OK;
}
}  // namespace

extern "C" int qsv_plan_create(qsv_state* s, int nblocks, const int* ks, const int* targets_flat,
                               const double* mats_c128, qsv_plan** out) {
  QSV_CHECK_HANDLE(s);
  if (!out) return set_error(s, QSV_ERR_INVALID, "null plan output");
  *out = nullptr;
  if (s->dtype != QSV_C64) return set_error(s, QSV_ERR_UNSUPPORTED, "fused blocks need a complex64 state");
  if (nblocks < 1 || !ks || !targets_flat || !mats_c128) return set_error(s, QSV_ERR_INVALID, "bad block list");
  auto* p = new (std::nothrow) qsv_plan();
  if (!p) return set_error(s, QSV_ERR_OOM, "host allocation failed");
  std::vector<size_t> img_off, mat_offs;
  size_t total = 0;
  int rc = prepare_blocks(s, nblocks, ks, targets_flat, p->args, img_off, mat_offs, total);
  if (rc) {
    delete p;
    return rc;
  }
  std::vector<uint8_t> host(total);
  for (int i = 0; i < nblocks; ++i)
    build_image(ks[i], mats_c128 + mat_offs[(size_t)i], p->args[(size_t)i].tperm, host.data() + img_off[(size_t)i],
                uses_interleaved_image(p->args[(size_t)i].mode));
  if (cudaMalloc(&p->d_images, total) != cudaSuccess) {
    cudaGetLastError();
    delete p;
    return set_error(s, QSV_ERR_OOM, "plan image allocation failed");
  }
  cudaError_t e = cudaMemcpy(p->d_images, host.data(), total, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(p->d_images);
    delete p;
    return set_error(s, QSV_ERR_CUDA, "plan upload: %s", cudaGetErrorString(e));
  }
  for (int i = 0; i < nblocks; ++i)
    p->args[(size_t)i].wimg = reinterpret_cast<const uint4*>((const uint8_t*)p->d_images + img_off[(size_t)i]);
  p->nblocks = nblocks;
  p->n = s->n;
  *out = p;
  return QSV_OK;
}

extern "C" int qsv_plan_launch(qsv_state* s, const qsv_plan* p, int first, int count) {
  QSV_CHECK_HANDLE(s);
  if (!p || first < 0 || count < 0 || first + count > p->nblocks)
    return set_error(s, QSV_ERR_INVALID, "bad plan range");
  if (p->n != s->n) return set_error(s, QSV_ERR_INVALID, "plan built for n=%d, state has n=%d", p->n, s->n);
  for (int i = first; i < first + count; ++i) {
    BlockArgs a = p->args[(size_t)i];
    a.flag = s->d_flag;
    int rc = launch_args(s, a);
    if (rc) return rc;
  }
  return QSV_OK;
}

extern "C" int qsv_inject_block_stall(qsv_state* s, uint64_t wait_ns) {
  QSV_CHECK_HANDLE(s);
  if (wait_ns < 1000 || wait_ns > 1000000000ull)
    return set_error(s, QSV_ERR_INVALID, "stall limit %llu ns outside [1 us, 1 s]", (unsigned long long)wait_ns);
  s->inject_stall_ns = wait_ns;
  return QSV_OK;
}

extern "C" int qsv_plan_destroy(qsv_plan* p) {
  if (!p) return QSV_OK;
  if (p->d_images) cudaFree(p->d_images);
  delete p;
  return QSV_OK;
}

extern "C" int qsv_apply_blocks(qsv_state* s, int nblocks, const int* ks, const int* targets_flat,
                                const double* mats_c128) {
  QSV_CHECK_HANDLE(s);
  if (s->dtype != QSV_C64) return set_error(s, QSV_ERR_UNSUPPORTED, "fused blocks need a complex64 state");
  if (nblocks < 0 || (nblocks > 0 && (!ks || !targets_flat || !mats_c128)))
    return set_error(s, QSV_ERR_INVALID, "bad block list");
  if (nblocks == 0) return QSV_OK;
  std::vector<BlockArgs> args;
  std::vector<size_t> img_off, mat_offs;
  size_t total = 0;
  int rc = prepare_blocks(s, nblocks, ks, targets_flat, args, img_off, mat_offs, total);
  if (rc) return rc;
  // Pinned staging slot from the ring: wait only if this slot's last upload is pending.
  const int slot = s->img_next;
  s->img_next = (slot + 1) % qsv_state::kImageSlots;
  if (!s->img_ev[slot]) QSV_CUDA(s, cudaEventCreateWithFlags(&s->img_ev[slot], cudaEventDisableTiming));
  if (s->img_busy[slot]) {
    QSV_CUDA(s, cudaEventSynchronize(s->img_ev[slot]));
    s->img_busy[slot] = false;
  }
  if (s->h_img_bytes[slot] < total) {
    if (s->h_img[slot]) cudaFreeHost(s->h_img[slot]);
    s->h_img[slot] = nullptr;
    s->h_img_bytes[slot] = 0;
    const size_t want = std::max(total, size_t(1) << 20);
    if (cudaMallocHost(&s->h_img[slot], want) != cudaSuccess) {
      cudaGetLastError();
      return set_error(s, QSV_ERR_OOM, "pinned staging allocation failed");
    }
    s->h_img_bytes[slot] = want;
  }
  if (s->d_images_bytes < total) {
    QSV_CUDA(s, cudaStreamSynchronize(s->stream));  // old images may still be in use
    if (s->d_images) cudaFree(s->d_images);
    s->d_images = nullptr;
    s->d_images_bytes = 0;
    const size_t want = std::max(total, size_t(4) << 20);
    if (cudaMalloc(&s->d_images, want) != cudaSuccess) {
      cudaGetLastError();
      return set_error(s, QSV_ERR_OOM, "device image allocation failed");
    }
    s->d_images_bytes = want;
  }
  uint8_t* himg = static_cast<uint8_t*>(s->h_img[slot]);
  for (int i = 0; i < nblocks; ++i)
    build_image(ks[i], mats_c128 + mat_offs[(size_t)i], args[(size_t)i].tperm, himg + img_off[(size_t)i],
                uses_interleaved_image(args[(size_t)i].mode));
  QSV_CUDA(s, cudaMemcpyAsync(s->d_images, himg, total, cudaMemcpyHostToDevice, s->stream));
  QSV_CUDA(s, cudaEventRecord(s->img_ev[slot], s->stream));
  s->img_busy[slot] = true;
  for (int i = 0; i < nblocks; ++i) {
    BlockArgs& a = args[(size_t)i];
    a.wimg = reinterpret_cast<const uint4*>((const uint8_t*)s->d_images + img_off[(size_t)i]);
    rc = launch_args(s, a);
    if (rc) return rc;
  }
  return QSV_OK;
}

// ---- batched launches for the tensor-core adjoint (qsv_adjtc.cu) ----------------------
namespace qsv {
struct FusedGeom {
  BlockArgs a;
  int low;  // targets among address bits 0..6
};

size_t fused_image_bytes(int k) { return image_bytes(k); }

int fused_geom_create(int device, int n, int k, const int* qubits, FusedGeom** out, uint8_t* tperm_out) {
  *out = nullptr;
  if (k < 4 || k > 6 || n - k < FB_BATCH_BITS) return QSV_ERR_INVALID;
  auto* g = new (std::nothrow) FusedGeom();
  if (!g) return QSV_ERR_OOM;
  int pos[8];
  int low = 0;
  for (int j = 0; j < k; ++j) {
    if (qubits[j] < 0 || qubits[j] >= n) {
      delete g;
      return QSV_ERR_INVALID;
    }
    pos[j] = n - 1 - qubits[j];
    if (pos[j] < FB_BATCH_BITS) low |= 1 << pos[j];
  }
  g->a = BlockArgs{};
  g->a.k = k;
  g->a.ntiles = 1ull << (n - k - FB_BATCH_BITS);
  g->low = low;
  tile_geometry(k, pos, g->a, lookup_mode(device, k, low));
  memcpy(tperm_out, g->a.tperm, 64);
  *out = g;
  return QSV_OK;
}

void fused_geom_destroy(FusedGeom* g) { delete g; }

bool fused_geom_interleaved(const FusedGeom* g) { return uses_interleaved_image(g->a.mode); }

bool fused_geom_backward_ok(const FusedGeom* g) {
  const int m = g->a.mode;
  return g->a.k == 6 && (m == MODE_DIRECT || m == MODE_PREFIX || m == MODE_PAIR1 || m == MODE_PAIR2);
}

template <int MODE>
cudaError_t launch_adj_back(const BlockArgs& g, const AdjBackArgs& a, unsigned grid, cudaStream_t stream) {
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(k_adj_back<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, AB_SMEM);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  k_adj_back<MODE><<<grid, AB_THREADS, AB_SMEM, stream>>>(g, a);
  return cudaGetLastError();
}

int fused_geom_launch_backward(const FusedGeom* geom, float2* psi, float2* lam, double* corr, int nsets, int n,
                               const void* images, size_t img_stride, int* flag, cudaStream_t stream, int sm_count) {
  if (!fused_geom_backward_ok(geom)) return QSV_ERR_UNSUPPORTED;
  AdjBackArgs a{};
  a.psi = psi;
  a.lam = lam;
  a.corr = corr;
  a.wimg = static_cast<const uint8_t*>(images);
  a.img_stride = img_stride;
  a.set_amps = 1ull << n;
  a.nsets = (uint64_t)nsets;
  a.flag = flag;
  // One CTA per SM (shared memory, all 512 TMEM columns).
  uint64_t grid = (uint64_t)std::max(1, sm_count);
  const uint64_t work = geom->a.ntiles * (uint64_t)nsets;
  if (grid > work) grid = work;
  cudaError_t e;
  switch (geom->a.mode) {
    case MODE_PREFIX: e = launch_adj_back<MODE_PREFIX>(geom->a, a, (unsigned)grid, stream); break;
    case MODE_PAIR1: e = launch_adj_back<MODE_PAIR1>(geom->a, a, (unsigned)grid, stream); break;
    case MODE_PAIR2: e = launch_adj_back<MODE_PAIR2>(geom->a, a, (unsigned)grid, stream); break;
    default: e = launch_adj_back<MODE_DIRECT>(geom->a, a, (unsigned)grid, stream); break;
  }
  if (e != cudaSuccess) return QSV_ERR_CUDA;
  count_launch();
  return QSV_OK;
}

int fused_geom_launch_sets(const FusedGeom* g, float2* psi, int nsets, int n, const void* images,
                           size_t img_stride, int* flag, cudaStream_t stream, int sm_count) {
  BlockArgs a = g->a;
  a.set_tiles = a.ntiles;
  a.set_amps = 1ull << n;
  a.ntiles = a.set_tiles * (uint64_t)nsets;
  a.img_stride = img_stride;
  a.wimg = static_cast<const uint4*>(images);
  a.flag = flag;
  a.wait_ns = FB_WAIT_NS;
  a.stall_first = 0;
  cudaError_t e;
  switch (a.k * 8 + a.mode) {
#define QSV_FB_CASE(KQ, MODE) \
  case KQ * 8 + MODE:         \
    e = launch_fb<KQ, MODE>(a, psi, stream, sm_count); \
    break;
    QSV_FB_CASE(4, MODE_DIRECT) QSV_FB_CASE(4, MODE_STAGED) QSV_FB_CASE(4, MODE_SHUF)
    QSV_FB_CASE(5, MODE_DIRECT) QSV_FB_CASE(5, MODE_STAGED) QSV_FB_CASE(5, MODE_SHUF)
    QSV_FB_CASE(6, MODE_DIRECT) QSV_FB_CASE(6, MODE_STAGED) QSV_FB_CASE(6, MODE_SHUF) QSV_FB_CASE(6, MODE_PREFIX)
    QSV_FB_CASE(6, MODE_PAIR1) QSV_FB_CASE(6, MODE_PAIR2)
#undef QSV_FB_CASE
    default: return QSV_ERR_INVALID;
  }
  if (e != cudaSuccess) return QSV_ERR_CUDA;
  count_launch();
  return QSV_OK;
}
}  // namespace qsv

namespace qsv {
int oob_take_fused(unsigned long long* count, unsigned long long* first) {
#ifdef QSV_BOUNDS_CHECK
  return qsv_oob_take_unit(count, first);
#else
  (void)count;
  (void)first;
  return 0;
#endif
}
}  // namespace qsv

// ---- access-mode autotuning --------------------------------------------------------------
extern "C" int qsv_set_block_mode(qsv_state* s, int k, int low_mask, int mode) {
  QSV_CHECK_HANDLE(s);
  if (k < 4 || k > 6 || low_mask < 0 || low_mask >= (1 << FB_BATCH_BITS) || __builtin_popcount(low_mask) > k)
    return set_error(s, QSV_ERR_INVALID, "bad placement class k=%d low_mask=%d", k, low_mask);
  if (mode < -1 || mode >= NUM_MODES) return set_error(s, QSV_ERR_INVALID, "bad access mode %d", mode);
  std::lock_guard<std::mutex> lk(g_mode_mu);
  if (mode < 0) {
    g_modes.erase(mode_key(s->device, k, low_mask));
    return QSV_OK;
  }
  if (!mode_applies(k, low_mask, mode))
    return set_error(s, QSV_ERR_INVALID, "mode %d does not apply to k=%d low_mask=%d", mode, k, low_mask);
  g_modes[mode_key(s->device, k, low_mask)] = mode;
  return QSV_OK;
}

extern "C" int qsv_tune_blocks(qsv_state* s, int count, const int* ks, const int* low_masks, int reps,
                               double* out_ms, int* out_mode) {
  QSV_CHECK_HANDLE(s);
  if (count < 0 || (count > 0 && (!ks || !low_masks || !out_ms || !out_mode)) || reps < 1 || reps > 1000)
    return set_error(s, QSV_ERR_INVALID, "bad tuning request");
  if (count == 0) return QSV_OK;
  const int nt = std::min(s->n, 26);
  for (int i = 0; i < count; ++i) {
    const int k = ks[i], low = low_masks[i];
    if (k < 4 || k > 6 || low < 0 || low >= (1 << FB_BATCH_BITS) || __builtin_popcount(low) > k)
      return set_error(s, QSV_ERR_INVALID, "class %d: bad placement k=%d low_mask=%d", i, k, low);
    if (nt - (k - __builtin_popcount(low)) < FB_BATCH_BITS || nt - k < FB_BATCH_BITS)
      return set_error(s, QSV_ERR_UNSUPPORTED, "class %d: n=%d too small to tune k=%d", i, s->n, k);
  }
  // Scratch state (zeros) and one identity image per k; the caller's state is untouched.
  float2* scratch = nullptr;
  uint8_t* dimg = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = QSV_OK;
  const size_t sbytes = sizeof(float2) << nt;
  const size_t ibytes = image_bytes(6);
  std::vector<uint8_t> himg(ibytes);
  std::vector<double> ident;
  // Identity images for k = 4, 5, 6 and the interleaved k = 6 image of the prefix mode.
  if (cudaMalloc(&scratch, sbytes) != cudaSuccess || cudaMalloc(&dimg, 4 * ibytes) != cudaSuccess) {
    cudaGetLastError();
    rc = set_error(s, QSV_ERR_OOM, "tuning scratch allocation failed");
  }
  if (!rc && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess))
    rc = set_error(s, QSV_ERR_CUDA, "event creation failed");
  if (!rc && cudaMemsetAsync(scratch, 0, sbytes, s->stream) != cudaSuccess)
    rc = set_error(s, QSV_ERR_CUDA, "scratch clear failed");
  for (int k = 4; k <= 6 && !rc; ++k) {
    const int T = 1 << k;
    ident.assign((size_t)2 * T * T, 0.0);
    for (int t = 0; t < T; ++t) ident[(size_t)2 * (t * T + t)] = 1.0;
    uint8_t idperm[64];
    for (int t = 0; t < T; ++t) idperm[t] = (uint8_t)t;
    build_image(k, ident.data(), idperm, himg.data());
    if (cudaMemcpy(dimg + (k - 4) * ibytes, himg.data(), image_bytes(k), cudaMemcpyHostToDevice) != cudaSuccess)
      rc = set_error(s, QSV_ERR_CUDA, "tuning image upload failed");
    if (k == 6 && !rc) {
      build_image(k, ident.data(), idperm, himg.data(), true);
      if (cudaMemcpy(dimg + 3 * ibytes, himg.data(), image_bytes(k), cudaMemcpyHostToDevice) != cudaSuccess)
        rc = set_error(s, QSV_ERR_CUDA, "tuning image upload failed");
    }
  }
  for (int i = 0; i < count && !rc; ++i) {
    const int k = ks[i], low = low_masks[i];
    int tpos[8], nt_pos = 0;
    for (int p = FB_BATCH_BITS - 1; p >= 0; --p)
      if ((low >> p) & 1) tpos[nt_pos++] = p;
    for (int p = nt - 1; nt_pos < k; --p) tpos[nt_pos++] = p;
    std::sort(tpos, tpos + k, [](int x, int y) { return x > y; });
    double best = -1.0;
    int best_mode = -1;
    for (int mode = 0; mode < NUM_MODES && !rc; ++mode) {
      out_ms[NUM_MODES * i + mode] = -1.0;
      if (!mode_applies(k, low, mode)) continue;
      BlockArgs a{};
      a.k = k;
      a.ntiles = 1ull << (nt - k - FB_BATCH_BITS);
      tile_geometry(k, tpos, a, mode);
      if (a.mode != mode) continue;
      a.flag = s->d_flag;
      a.wimg = reinterpret_cast<const uint4*>(dimg + (uses_interleaved_image(mode) ? 3 : k - 4) * ibytes);
      rc = launch_args_on(s, a, scratch);
      if (!rc && cudaEventRecord(e0, s->stream) != cudaSuccess) rc = set_error(s, QSV_ERR_CUDA, "event record");
      for (int r = 0; r < reps && !rc; ++r) rc = launch_args_on(s, a, scratch);
      if (!rc && cudaEventRecord(e1, s->stream) != cudaSuccess) rc = set_error(s, QSV_ERR_CUDA, "event record");
      float ms = 0.0f;
      if (!rc && (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
        rc = set_error(s, QSV_ERR_CUDA, "tuning timing failed");
      if (rc) break;
      const double per = (double)ms / reps;
      out_ms[NUM_MODES * i + mode] = per;
      if (best < 0.0 || per < best) {
        best = per;
        best_mode = mode;
      }
    }
    out_mode[i] = best_mode;
    if (!rc && best_mode >= 0) {
      std::lock_guard<std::mutex> lk(g_mode_mu);
      g_modes[mode_key(s->device, k, low)] = best_mode;
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (scratch || dimg) {
    cudaStreamSynchronize(s->stream);
    if (scratch) cudaFree(scratch);
    if (dimg) cudaFree(dimg);
  }
  return rc;
}
