// Adjoint gradients on the tensor cores (no reference counterpart: the reference has no
// gradients).
//
// Circuit: rotations RY(theta) = exp(-i theta Y/2), RZ(theta) = exp(-i theta Z/2) and
// CNOTs on n qubits, for a batch of nsets parameter sets (one state of 2^n complex64
// amplitudes per set, back to back).  The host splits the gate list into blocks of six
// qubits (the fusion planner's order, a valid order of the circuit).
//
// Forward: per block, k_adj_images builds every set's 64x64 block matrix U from its
// angles and writes its bf16 hi/lo W image; one fused-block launch (k_block_tc over all
// sets, each with its own W) applies it.  Backward (adjoint method, no checkpoints):
// with psi = psi_out and lambda = lambda_out at a block's end,
//     dE/dtheta_j = Im <lambda_j| P_j |psi_j> = Im Tr(P_j Q_j),
//     Q_m = X = sum_g psi_out[g] lambda_out[g]^+   (64 x 64 per set),
//     Q_{j-1} = U_j^+ Q_j U_j,
// over the block's gates j = m..1 (g runs over the 2^(n-6) groups of the other qubits,
// A_j = U_m..U_{j+1}, psi_j = A_j^+ psi_out, lambda_j = A_j^+ lambda_out, so the sum
// over groups is Tr(A_j P_j A_j^+ X) = Tr(P_j Q_j)).  For blocks in the direct, prefix
// and pair access modes one launch (k_adj_back, qsv_fused.cu) un-computes psi and lambda
// with U^+ and computes X on the tensor cores from the same operand images; for the
// others k_adj_corr_d computes X as a real GEMM (K = the groups) and two fused-block
// launches un-compute psi and lambda.  k_adj_walk then walks Q through the block's gates
// in FP64 and writes the gradients.  Every block's gradients cost one pass over psi and
// lambda instead of a pass per gate.
//
// Local index convention: a block's qubits q_0 < ... < q_5; bit 5-j of a local index
// (matrix row/column, X's indices) is qubit q_j, whose address bit is n-1-q_j.

#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "qsv_internal.cuh"
#include "qsv_tc.cuh"

using namespace qsv;

namespace {

constexpr int AK = 6;               // qubits per block
constexpr int AT = 1 << AK;         // 64 local indices
constexpr int AKD = 2 * AT;         // 128: [Re | Im]
constexpr int A_THREADS = 256;
constexpr int CORR_K = 64;          // groups per correlation tile (the GEMM's K)
constexpr int CORR_OP_BYTES = AKD * CORR_K * 2;  // one bf16 operand image (16 KiB)
constexpr int CORR_GROUPS = 8;                        // sets read concurrently
constexpr int CORR_THREADS = 512;                     // 16 warps: four 4-group runs per thread
constexpr int GATE_RY = 0, GATE_RZ = 1, GATE_CNOT = 2;

// A gate of a block: kind, local target bit, local control bit (-1), parameter index.
struct AdjGate {
  int kind, t, c, param;
};

struct AdjBlockDev {
  int first_gate, ngates;
  int interleaved;     // W image rows interleaved [Re t', Im t'] (the block kernel's prefix mode)
  uint64_t dept[AT];   // address offset of local index t
  int tpos[AK];        // the block's bit positions, ascending (a group index gets zeros there)
  uint8_t tperm[64];   // fused kernel's target order -> local index
};

__device__ __forceinline__ void rot_matrix(int kind, double th, double2* u) {
  if (kind == GATE_RY) {
    double s, c;
    sincos(0.5 * th, &s, &c);
    u[0] = make_double2(c, 0.0);
    u[1] = make_double2(-s, 0.0);
    u[2] = make_double2(s, 0.0);
    u[3] = make_double2(c, 0.0);
  } else {
    double s, c;
    sincos(0.5 * th, &s, &c);
    u[0] = make_double2(c, -s);
    u[1] = make_double2(0.0, 0.0);
    u[2] = make_double2(0.0, 0.0);
    u[3] = make_double2(c, s);
  }
}

__device__ __forceinline__ uint16_t bf16_bits(float f) {
  __nv_bfloat16 h = __float2bfloat16_rn(f);
  return *reinterpret_cast<uint16_t*>(&h);
}

// ---- per-set block images ------------------------------------------------------------
// grid = nsets.  U (FP32, 64x64 complex) is built in shared memory from the identity by
// the block's gates in order (rows: U <- G U), then the W image of U (or of U^+ with
// DAGGER) is written in the fused kernel's layout: W = [[Mr, -Mi], [Mi, Mr]] read at
// (tperm[nn % 64], tperm[kk % 64]), element (nn, kk) at (kk/8)*(128*16) + nn*16 + (kk%8)*2
// bytes, hi image then lo image (x = hi + lo, both bf16).
template <bool DAGGER>
__global__ void __launch_bounds__(A_THREADS)
    k_adj_images(const AdjBlockDev* __restrict__ blk, const AdjGate* __restrict__ gates,
                 const double* __restrict__ thetas, int nparams, uint8_t* __restrict__ images,
                 size_t img_stride) {
  __shared__ float2 U[AT][AT];
  __shared__ uint8_t tperm[64];
  const int tid = threadIdx.x;
  const int set = blockIdx.x;
  const bool inter = blk->interleaved != 0;
  for (int i = tid; i < AT * AT; i += A_THREADS) U[i / AT][i % AT] = make_float2((i / AT) == (i % AT) ? 1.f : 0.f, 0.f);
  if (tid < 64) tperm[tid] = blk->tperm[tid];
  __syncthreads();
  for (int g = 0; g < blk->ngates; ++g) {
    const AdjGate G = gates[blk->first_gate + g];
    const int tb = 1 << G.t;
    if (G.kind == GATE_CNOT) {
      const int cb = 1 << G.c;
      // Swap rows r and r^tb where the control bit is 1: 16 row pairs x 64 columns.
      for (int i = tid; i < 16 * AT; i += A_THREADS) {
        const int col = i % AT, p = i / AT;  // p: 4 free bits
        int r = 0;
        for (int b = 0, k = 0; b < AK; ++b) {
          if ((1 << b) == tb) continue;
          if ((1 << b) == cb) {
            r |= cb;
            continue;
          }
          if ((p >> k++) & 1) r |= 1 << b;
        }
        const float2 x = U[r][col];
        U[r][col] = U[r | tb][col];
        U[r | tb][col] = x;
      }
    } else {
      double2 ud[4];
      rot_matrix(G.kind, thetas[(size_t)set * nparams + G.param], ud);
      float2 u[4];
      for (int i = 0; i < 4; ++i) u[i] = make_float2((float)ud[i].x, (float)ud[i].y);
      for (int i = tid; i < 32 * AT; i += A_THREADS) {
        const int col = i % AT, p = i / AT;  // p: the 5 other bits
        const int r0 = ((p >> G.t) << (G.t + 1)) | (p & (tb - 1));
        const float2 a = U[r0][col], b = U[r0 | tb][col];
        U[r0][col] = qsv_cfma(u[1], b, qsv_cmul(u[0], a));
        U[r0 | tb][col] = qsv_cfma(u[3], b, qsv_cmul(u[2], a));
      }
    }
    __syncthreads();
  }
  uint16_t* hi = reinterpret_cast<uint16_t*>(images + (size_t)set * img_stride);
  uint16_t* lo = hi + AKD * AKD;
  // Items (nn, kk/8): 8 consecutive kk are one 16-byte row of a core matrix.
  for (int item = tid; item < AKD * (AKD / 8); item += A_THREADS) {
    const int nn = item % AKD, k8 = item / AKD;
    const int tp = tperm[inter ? nn >> 1 : nn % AT];
    const bool out_im = inter ? (nn & 1) != 0 : nn >= AT;
    uint16_t h[8], l[8];
    for (int q = 0; q < 8; ++q) {
      const int kk = k8 * 8 + q;
      const int t = tperm[kk % AT];
      const bool in_im = kk >= AT;
      float2 m = DAGGER ? make_float2(U[t][tp].x, -U[t][tp].y) : U[tp][t];
      const float w = out_im ? (in_im ? m.x : m.y) : (in_im ? -m.y : m.x);
      h[q] = bf16_bits(w);
      const float hv = __uint_as_float((uint32_t)h[q] << 16);
      l[q] = bf16_bits(w - hv);
    }
    const size_t e = (size_t)k8 * (AKD * 8) + (size_t)nn * 8;
    uint4 vh, vl;
    vh.x = h[0] | ((uint32_t)h[1] << 16);
    vh.y = h[2] | ((uint32_t)h[3] << 16);
    vh.z = h[4] | ((uint32_t)h[5] << 16);
    vh.w = h[6] | ((uint32_t)h[7] << 16);
    vl.x = l[0] | ((uint32_t)l[1] << 16);
    vl.y = l[2] | ((uint32_t)l[3] << 16);
    vl.z = l[4] | ((uint32_t)l[5] << 16);
    vl.w = l[6] | ((uint32_t)l[7] << 16);
    *reinterpret_cast<uint4*>(hi + e) = vh;
    *reinterpret_cast<uint4*>(lo + e) = vl;
  }
}

// ---- correlation X = sum_g psi[g] lambda[g]^+ on the tensor cores ----------------------
// One real GEMM per tile of 64 groups: D[m][nn] = sum_k A[m][k] B[nn][k] with A rows
// m = (Re psi_t | Im psi_t), B rows nn = (Re lambda_t | Im lambda_t), k = group, split-bf16
// (hi*lo + lo*hi + hi*hi) with FP32 accumulation in TMEM, a fresh accumulator per tile
// (12 accumulating MMA steps).  Each thread adds its 64 entries of every tile into FP32
// registers (round to nearest) and flushes them with FP64 atomics into corr[set][m][nn]
// whenever its next tile belongs to another set, and at the end.  Then
// X[b][a] = D[b][a] + D[64+b][64+a] + i (D[64+b][a] - D[b][64+a]).
// Tiles go to CTAs grid-stride (tile = blockIdx.x + i * gridDim.x), so the CTAs running
// at one time read neighbouring memory, as the fused block kernel does; a CTA then meets
// every set once and flushes once per set.
//
// Loads: a tile is, for each state (psi, lambda) and local index t, 64 groups; threads
// read aligned 32-byte runs straight into registers (k_adj_corr_d below, one variant per
// role of address bits 0 and 1).
//
// Order: the CTAs form CORR_GROUPS groups; group q takes sets q, q + CORR_GROUPS, ... and
// its CTAs stride through each set's tiles together, so concurrent reads stay close in
// memory and a CTA flushes its sums once per set it visits.
struct CorrArgs {
  const float2* psi;
  const float2* lam;
  double* corr;       // [nsets][128][128]
  uint64_t ntiles;    // nsets * 2^(n-12)
  int tile_shift;     // log2(tiles per set) = n - 12
  int n;
  uint64_t set_amps;  // 2^n
  int* flag;
  const AdjBlockDev* blk;
};

// The correlation kernel.  Each thread loads 4 aligned 32-byte runs (4 consecutive
// amplitudes) of a tile into registers and writes 4 runs (state, t, groups 4*g4 ..
// 4*g4+3) into the operand images as 8-byte chunks.  There is no staging buffer: an
// earlier version that staged tiles through shared memory with cp.async moved three
// times the shared bytes.  Two tiles live in registers: tile i+2's loads are issued while
// tile i's products run, so every tile's reads have a whole iteration to land.  The
// running sums sit in TMEM columns 128..255 next to the products (added in registers,
// round to nearest, and stored back), which leaves the registers for the second tile.
//  LM = 0, no target on address bits 0, 1: a 32-byte run is 4 groups of one t.  Warp w
//    takes state w/8, t = 8*(w%8) + lane/4, run g4 = lane%4 + 4u (u = 0..3): 128
//    contiguous bytes per t and load.
//  LM = 1, targets on address bits 0 and 1 (t bits 0, 1): a run is 4 targets of one
//    group.  Loads: lane bits 0, 1 = group bits 0, 1, lane bits 2, 3 = t bits 2, 3, lane
//    bit 4 = group bit 2, warp bits 0, 1 = t bits 4, 5, warp bit 2 = group bit 3, warp bit
//    3 = state, u = group bits 4, 5 (4 lanes read 128 contiguous bytes for every such
//    placement).  A 4 x 4 transpose over lane bits 0, 1 (two shfl.xor rounds) then
//    gives each thread 4 groups of one t per run: t = lane%16 + 16*(w%4),
//    g4 = lane/16 + 2*((w/4)%2) + 4u.
//  LM = 2 / 3, one target and one group bit on address bits 0, 1 (LM = 2: t bit 0 on
//    address bit 0; LM = 3: group bit 0 there): a run is 2 targets x 2 groups.  Loads:
//    lane bit 0 = group bit 1, lane bits 1, 2 = t bits 1, 2, lane bit 3 = group bit 2, lane
//    bit 4 = t bit 3, warp bits 0, 1 = t bits 4, 5, warp bit 2 = group bit 3, u = group
//    bits 4, 5.  After putting group bit 0 in register bit 0 (LM = 2 swaps registers 1
//    and 2), one shfl.xor round over lane bit 0 trades t bit 0 for group bit 1.
// Every mode's 8-byte operand stores of a warp fill 16 distinct bank slots.
// A hi/lo, B hi/lo, then the mbarrier, the TMEM slot and the abort flag.
constexpr int CORRD_SMEM = 4 * CORR_OP_BYTES + 64;

template <int LM>
__global__ void __launch_bounds__(CORR_THREADS, 1) k_adj_corr_d(const __grid_constant__ CorrArgs a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sA_hi = smem;
  uint8_t* sA_lo = smem + CORR_OP_BYTES;
  uint8_t* sB_hi = smem + 2 * CORR_OP_BYTES;
  uint8_t* sB_lo = smem + 3 * CORR_OP_BYTES;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + 4 * CORR_OP_BYTES);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mbar + 1);
  int* abort_flag = reinterpret_cast<int*>(tmem_slot + 1);
  __shared__ uint64_t dept[AT];
  __shared__ int tpos[AK];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int i = tid; i < AT; i += CORR_THREADS) dept[i] = a.blk->dept[i];
  if (tid < AK) tpos[tid] = a.blk->tpos[tid];
  if (tid == 0) {
    mbar_init(smem_u32(mbar), 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"((uint32_t)(2 * AKD))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  // This CTA's tiles: group grp of the CTAs, rank within the group.
  const uint64_t nsets = a.ntiles >> a.tile_shift;
  const uint64_t tps = 1ull << a.tile_shift;
  uint64_t ngr64 = nsets < (uint64_t)gridDim.x ? nsets : (uint64_t)gridDim.x;
  if (ngr64 > (uint64_t)CORR_GROUPS) ngr64 = CORR_GROUPS;
  const int ngr = (int)ngr64;
  const int grp = blockIdx.x % ngr;
  const uint64_t rank = blockIdx.x / ngr;
  const uint64_t nctas = (gridDim.x - grp + ngr - 1) / ngr;
  const uint64_t cnt = rank < tps ? (tps - rank + nctas - 1) / nctas : 0;
  const uint64_t nsg = (nsets - grp + ngr - 1) / ngr;
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
  auto tile_of = [&](const Pos& p) -> uint64_t { return (p.set << a.tile_shift) + p.local; };

  const int state = warp >> 3;
  const float2* src = state ? a.lam : a.psi;
  // The run each thread writes: local index t, run g4_of(u).
  const int t = LM == 0   ? ((warp & 7) << 3) | (lane >> 2)
                : LM == 1 ? (lane & 15) | ((warp & 3) << 4)
                          : (lane & 7) | (((lane >> 4) & 1) << 3) | ((warp & 3) << 4);
  auto g4_of = [&](int u) -> int {
    return LM == 0   ? (lane & 3) | (u << 2)
           : LM == 1 ? (lane >> 4) | (((warp >> 2) & 1) << 1) | (u << 2)
                     : ((lane >> 3) & 1) | (((warp >> 2) & 1) << 1) | (u << 2);
  };
  // Address offset of load u within a tile: local index and group of its first amplitude.
  uint64_t off[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    int tl, gl;
    if (LM == 0) {
      tl = t;
      gl = 4 * g4_of(u);
    } else if (LM == 1) {
      tl = (lane & 12) | ((warp & 3) << 4);
      gl = (lane & 3) | (((lane >> 4) & 1) << 2) | (((warp >> 2) & 1) << 3) | (u << 4);
    } else {
      tl = (lane & 6) | (((lane >> 4) & 1) << 3) | ((warp & 3) << 4);
      gl = ((lane & 1) << 1) | (((lane >> 3) & 1) << 2) | (((warp >> 2) & 1) << 3) | (u << 4);
    }
    off[u] = dept[tl] + qsv_insert_zeros((uint64_t)gl, tpos, AK);
  }
  [[maybe_unused]] const uint64_t lim = a.set_amps * nsets;
  float2 buf0[4][4], buf1[4][4];
  auto load = [&](uint64_t tile, float2 (&buf)[4][4]) {
    const uint64_t set = tile >> a.tile_shift;
    const uint64_t row = set * a.set_amps + qsv_insert_zeros((tile & (tps - 1)) << 6, tpos, AK);
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (QSV_IN_BOUNDS(row + off[u] + 3, lim)) ld_v8(src + row + off[u], buf[u]);
  };
  constexpr int LBO = AKD * 16;  // K-step between core matrices (both operands: 128 rows)
  auto write_ops = [&](float2 (&buf)[4][4]) {
    uint8_t* hi = state ? sB_hi : sA_hi;
    uint8_t* lo = state ? sB_lo : sA_lo;
    if constexpr (LM == 1) {
      // buf[u][j]: t bits 0, 1 = j, group bits 0, 1 = lane bits 0, 1.  Swap the two roles.
#pragma unroll
      for (int b = 0; b < 2; ++b) {
        const bool up = (lane >> b) & 1;
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            if (j & (1 << b)) continue;
            const int j1 = j | (1 << b);
            const float2 send = up ? buf[u][j] : buf[u][j1];
            float2 got;
            got.x = __shfl_xor_sync(0xffffffffu, send.x, 1 << b);
            got.y = __shfl_xor_sync(0xffffffffu, send.y, 1 << b);
            if (up)
              buf[u][j] = got;
            else
              buf[u][j1] = got;
          }
      }
    } else if constexpr (LM >= 2) {
      // Register bit 0 = group bit 0, bit 1 = t bit 0 (LM = 2 loads them the other way
      // round); then trade t bit 0 (register bit 1) for group bit 1 (lane bit 0).
      const bool up = lane & 1;
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if constexpr (LM == 2) {
          const float2 x = buf[u][1];
          buf[u][1] = buf[u][2];
          buf[u][2] = x;
        }
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          const float2 send = up ? buf[u][j] : buf[u][j + 2];
          float2 got;
          got.x = __shfl_xor_sync(0xffffffffu, send.x, 1);
          got.y = __shfl_xor_sync(0xffffffffu, send.y, 1);
          if (up)
            buf[u][j] = got;
          else
            buf[u][j + 2] = got;
        }
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int g4 = g4_of(u);
      float re[4], im[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        re[j] = buf[u][j].x;
        im[j] = buf[u][j].y;
      }
      uint2 rh, rl, ih, il;
      split4(re, rh, rl);
      split4(im, ih, il);
      // Row t (Re) / AT + t (Im), K = groups 4*g4 .. 4*g4+3 of the tile.
      const uint32_t off_re = (uint32_t)(g4 >> 1) * LBO + (uint32_t)t * 16 + (uint32_t)(g4 & 1) * 8;
      const uint32_t off_im = off_re + AT * 16;
      *reinterpret_cast<uint2*>(hi + off_re) = rh;
      *reinterpret_cast<uint2*>(lo + off_re) = rl;
      *reinterpret_cast<uint2*>(hi + off_im) = ih;
      *reinterpret_cast<uint2*>(lo + off_im) = il;
    }
  };
  constexpr uint32_t idesc = make_idesc(AKD, AKD);
  auto issue = [&]() {
    if (tid == 0) {
      const uint32_t ah = smem_u32(sA_hi), al = smem_u32(sA_lo), bh = smem_u32(sB_hi), bl = smem_u32(sB_lo);
      constexpr int KSTEPS = CORR_K / 16;
#pragma unroll
      for (int s = 0; s < KSTEPS; ++s)
        tc_mma(tmem, make_smem_desc(ah + s * 2 * LBO, LBO, 128), make_smem_desc(bl + s * 2 * LBO, LBO, 128), idesc,
               s > 0 ? 1u : 0u);
#pragma unroll
      for (int s = 0; s < KSTEPS; ++s)
        tc_mma(tmem, make_smem_desc(al + s * 2 * LBO, LBO, 128), make_smem_desc(bh + s * 2 * LBO, LBO, 128), idesc, 1u);
#pragma unroll
      for (int s = 0; s < KSTEPS; ++s)
        tc_mma(tmem, make_smem_desc(ah + s * 2 * LBO, LBO, 128), make_smem_desc(bh + s * 2 * LBO, LBO, 128), idesc, 1u);
      tc_commit(smem_u32(mbar));
    }
  };
  // This thread's TMEM lane (row 32q + lane) and 32 columns: the tile's products at
  // taddr, the running sums AKD columns further.
  const int q = warp & 3, h = warp >> 2;
  const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(h * 32);
  const uint32_t saddr = taddr + AKD;
  auto zero_sums = [&]() {
    float z[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) z[k] = 0.f;
    tmem_st16(saddr, z);
    tmem_st16(saddr + 16, z);
    tmem_st_wait();
  };
  auto flush = [&](uint64_t set) {
    double* dst = a.corr + set * (uint64_t)(AKD * AKD) + (uint64_t)(q * 32 + lane) * AKD + h * 32;
#pragma unroll
    for (int c = 0; c < 32; c += 16) {
      float sv[16];
      tmem_ld<16>(saddr + (uint32_t)c, sv);
      tmem_ld_wait();
#pragma unroll
      for (int k = 0; k < 16; ++k)
        if (sv[k] != 0.f) atomicAdd(dst + c + k, (double)sv[k]);
    }
    zero_sums();
  };
  uint32_t phase = 0;
  bool pending = false;
  Pos cu{(uint64_t)grp, rank, 0}, pf = cu;
  if (total > 0) load(tile_of(pf), buf0);
  advance(pf);
  if (total > 1) load(tile_of(pf), buf1);
  advance(pf);
  zero_sums();
  // Tile i (in buf, loaded an iteration or two ago); buf then takes tile i + 2.
  auto step = [&](uint64_t i, float2 (&buf)[4][4]) -> bool {
    write_ops(buf);
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    issue();
    pending = true;
    if (i + 2 < total) load(tile_of(pf), buf);
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
      return false;
    }
#pragma unroll
    for (int c = 0; c < 32; c += 16) {
      float d[16], sv[16];
      tmem_ld<16>(taddr + (uint32_t)c, d);
      tmem_ld<16>(saddr + (uint32_t)c, sv);
      tmem_ld_wait();
#pragma unroll
      for (int k = 0; k < 16; ++k) sv[k] += d[k];
      tmem_st16(saddr + (uint32_t)c, sv);
    }
    tmem_st_wait();
    tc_fence_before();
    const uint64_t set = cu.set;
    advance(cu);
    if (cu.li == 0) flush(set);
    return true;
  };
  for (uint64_t i = 0; i < total;) {
    if (!step(i, buf0) || ++i >= total) break;
    if (!step(i, buf1)) break;
    ++i;
  }
  __syncthreads();
  if (*abort_flag) {
    if (pending) mbar_wait_bounded(smem_u32(mbar), phase);
    if (tid == 0) atomicExch(a.flag, 2);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)(2 * AKD))
                 : "memory");
  }
}

// ---- the gradient walk -----------------------------------------------------------------
// One launch for every block of the backward: grid = (nsets, nblocks), CTA (s, b) walks
// block b for set s from corr[b][s] (each block has its own correlation slice, so the walks
// are independent).  Q = X; for the block's gates from last to first: a rotation adds
// Im Tr(P Q) to its parameter's gradient (P = Y for RY, Z for RZ, on the gate's local bit;
// FP64 atomics, as gates of several blocks may share a parameter), then Q <- U^+ Q U.
__global__ void __launch_bounds__(A_THREADS)
    k_adj_walk(const AdjBlockDev* __restrict__ blocks, const AdjGate* __restrict__ gates,
               const double* __restrict__ thetas, int nparams, const double* __restrict__ corr,
               double* __restrict__ grads, int grad_stride) {
  extern __shared__ __align__(16) uint8_t wsm[];
  double2(*Q)[AT] = reinterpret_cast<double2(*)[AT]>(wsm);
  __shared__ double red[32];
  const int tid = threadIdx.x;
  const int set = blockIdx.x;
  const AdjBlockDev* blk = blocks + blockIdx.y;
  const double* D = corr + ((size_t)blockIdx.y * gridDim.x + set) * AKD * AKD;
  for (int i = tid; i < AT * AT; i += A_THREADS) {
    const int b = i / AT, c = i % AT;
    const double re = D[b * AKD + c] + D[(AT + b) * AKD + AT + c];
    const double im = D[(AT + b) * AKD + c] - D[b * AKD + AT + c];
    Q[b][c] = make_double2(re, im);
  }
  __syncthreads();
  for (int g = blk->ngates - 1; g >= 0; --g) {
    const AdjGate G = gates[blk->first_gate + g];
    const int tb = 1 << G.t;
    if (G.kind != GATE_CNOT) {
      // Im Tr(P Q): Z -> sum_r z_r Im Q[r][r]; Y -> sum_{r0} Re Q[r0][r1] - Re Q[r1][r0].
      double part = 0.0;
      if (tid < 64) {
        if (G.kind == GATE_RZ) {
          part = (tid & tb) ? -Q[tid][tid].y : Q[tid][tid].y;
        } else if (!(tid & tb)) {
          part = Q[tid][tid | tb].x - Q[tid | tb][tid].x;
        }
      }
      if (tid < 64) {
        for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
        if ((tid & 31) == 0) red[tid >> 5] = part;
      }
      __syncthreads();
      if (tid == 0) atomicAdd(&grads[(size_t)set * grad_stride + G.param], red[0] + red[1]);
      // U^+ Q U for the rotation u.
      double2 u[4];
      rot_matrix(G.kind, thetas[(size_t)set * nparams + G.param], u);
      const double2 d0 = make_double2(u[0].x, -u[0].y), d1 = make_double2(u[2].x, -u[2].y);
      const double2 d2 = make_double2(u[1].x, -u[1].y), d3 = make_double2(u[3].x, -u[3].y);
      for (int i = tid; i < 32 * AT; i += A_THREADS) {  // rows: Q <- u^+ Q
        const int col = i % AT, p = i / AT;
        const int r0 = ((p >> G.t) << (G.t + 1)) | (p & (tb - 1));
        const double2 a0 = Q[r0][col], a1 = Q[r0 | tb][col];
        Q[r0][col] = qsv_cfma(d1, a1, qsv_cmul(d0, a0));
        Q[r0 | tb][col] = qsv_cfma(d3, a1, qsv_cmul(d2, a0));
      }
      __syncthreads();
      for (int i = tid; i < 32 * AT; i += A_THREADS) {  // columns: Q <- Q u
        const int row = i % AT, p = i / AT;
        const int c0 = ((p >> G.t) << (G.t + 1)) | (p & (tb - 1));
        const double2 a0 = Q[row][c0], a1 = Q[row][c0 | tb];
        Q[row][c0] = qsv_cfma(a1, u[2], qsv_cmul(a0, u[0]));
        Q[row][c0 | tb] = qsv_cfma(a1, u[3], qsv_cmul(a0, u[1]));
      }
      __syncthreads();
    } else {
      // CNOT = its own inverse: swap rows, then columns, r <-> r ^ tb where bit c is 1.
      const int cb = 1 << G.c;
      for (int i = tid; i < 16 * AT; i += A_THREADS) {
        const int col = i % AT, p = i / AT;
        int r = cb;
        for (int b = 0, k = 0; b < AK; ++b) {
          if ((1 << b) == tb || (1 << b) == cb) continue;
          if ((p >> k++) & 1) r |= 1 << b;
        }
        const double2 x = Q[r][col];
        Q[r][col] = Q[r | tb][col];
        Q[r | tb][col] = x;
      }
      __syncthreads();
      for (int i = tid; i < 16 * AT; i += A_THREADS) {
        const int row = i % AT, p = i / AT;
        int c = cb;
        for (int b = 0, k = 0; b < AK; ++b) {
          if ((1 << b) == tb || (1 << b) == cb) continue;
          if ((p >> k++) & 1) c |= 1 << b;
        }
        const double2 x = Q[row][c];
        Q[row][c] = Q[row][c | tb];
        Q[row][c | tb] = x;
      }
      __syncthreads();
    }
  }
}

}  // namespace

struct qsv_adjoint_plan {
  int n = 0;
  int device = 0;
  int sm_count = 0;
  int nblocks = 0;
  int ngates = 0;
  int max_param = -1;
  std::vector<FusedGeom*> geom;
  // Correlation kernel of block b: k_adj_corr_d<kind>, by the roles of address bits 0, 1
  // (0: both group bits, 1: both target bits, 2: target, group, 3: group, target).
  std::vector<char> corr_kind;
  AdjBlockDev* d_blocks = nullptr;
  AdjGate* d_gates = nullptr;
  int* d_flag = nullptr;
};

namespace {
size_t image_stride() { return (fused_image_bytes(AK) + 255) / 256 * 256; }

int check_stream_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(nullptr, QSV_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  count_launch();
  return QSV_OK;
}
}  // namespace

extern "C" int qsv_adjoint_plan_create(int n, int nblocks, const int* block_qubits, const int* block_ngates,
                                       const int* gates, qsv_adjoint_plan** out) {
  if (!out) return set_error(nullptr, QSV_ERR_INVALID, "null plan output");
  *out = nullptr;
  if (n < AK + 7 || n > 34) return set_error(nullptr, QSV_ERR_UNSUPPORTED, "tensor-core adjoint needs 13 <= n <= 34");
  if (nblocks < 1 || nblocks > 65535 || !block_qubits || !block_ngates || !gates)
    return set_error(nullptr, QSV_ERR_INVALID, "bad plan (1..65535 blocks)");
  auto* p = new (std::nothrow) qsv_adjoint_plan();
  if (!p) return set_error(nullptr, QSV_ERR_OOM, "host allocation failed");
  p->n = n;
  p->nblocks = nblocks;
  cudaGetDevice(&p->device);
  cudaDeviceGetAttribute(&p->sm_count, cudaDevAttrMultiProcessorCount, p->device);
  std::vector<AdjBlockDev> hb((size_t)nblocks);
  std::vector<AdjGate> hg;
  int gofs = 0;
  for (int b = 0; b < nblocks; ++b) {
    const int* qs = block_qubits + AK * b;
    AdjBlockDev& B = hb[(size_t)b];
    memset(&B, 0, sizeof(B));
    uint64_t tmask = 0;
    for (int j = 0; j < AK; ++j) {
      if (qs[j] < 0 || qs[j] >= n || (j > 0 && qs[j] <= qs[j - 1])) {
        qsv_adjoint_plan_destroy(p);
        return set_error(nullptr, QSV_ERR_INVALID, "block %d: qubits must be ascending, distinct, in [0, n)", b);
      }
      tmask |= 1ull << (n - 1 - qs[j]);
    }
    for (int t = 0; t < AT; ++t) {
      uint64_t off = 0;
      for (int j = 0; j < AK; ++j)
        if ((t >> (AK - 1 - j)) & 1) off |= 1ull << (n - 1 - qs[j]);
      B.dept[t] = off;
    }
    for (int pbit = 0, k = 0; pbit < n; ++pbit)
      if ((tmask >> pbit) & 1) B.tpos[k++] = pbit;
    FusedGeom* g = nullptr;
    uint8_t tperm[64];
    if (fused_geom_create(p->device, n, AK, qs, &g, tperm) != QSV_OK) {
      qsv_adjoint_plan_destroy(p);
      return set_error(nullptr, QSV_ERR_INVALID, "block %d: no tile geometry", b);
    }
    p->geom.push_back(g);
    p->corr_kind.push_back(B.tpos[0] >= 2 ? 0 : B.tpos[0] == 1 ? 3 : B.tpos[1] == 1 ? 1 : 2);
    memcpy(B.tperm, tperm, 64);
    B.interleaved = fused_geom_interleaved(g) ? 1 : 0;
    B.first_gate = gofs;
    B.ngates = block_ngates[b];
    for (int i = 0; i < block_ngates[b]; ++i) {
      const int* G = gates + 4 * (size_t)(gofs + i);
      auto local = [&](int qubit) -> int {
        for (int j = 0; j < AK; ++j)
          if (qs[j] == qubit) return AK - 1 - j;
        return -1;
      };
      AdjGate a{G[0], local(G[1]), G[2] >= 0 ? local(G[2]) : -1, G[3]};
      const bool ok = (a.kind == GATE_RY || a.kind == GATE_RZ) ? (a.t >= 0 && a.param >= 0)
                                                             : (a.kind == GATE_CNOT && a.t >= 0 && a.c >= 0 && a.c != a.t);
      if (!ok) {
        qsv_adjoint_plan_destroy(p);
        return set_error(nullptr, QSV_ERR_INVALID, "block %d gate %d: bad kind, qubits or parameter", b, i);
      }
      p->max_param = std::max(p->max_param, a.param);
      hg.push_back(a);
    }
    gofs += block_ngates[b];
  }
  p->ngates = gofs;
  if (cudaMalloc(&p->d_blocks, hb.size() * sizeof(AdjBlockDev)) != cudaSuccess ||
      cudaMalloc(&p->d_gates, std::max<size_t>(1, hg.size()) * sizeof(AdjGate)) != cudaSuccess ||
      cudaMalloc(&p->d_flag, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    qsv_adjoint_plan_destroy(p);
    return set_error(nullptr, QSV_ERR_OOM, "plan tables: device allocation failed");
  }
  if (cudaMemcpy(p->d_blocks, hb.data(), hb.size() * sizeof(AdjBlockDev), cudaMemcpyHostToDevice) != cudaSuccess ||
      (hg.size() && cudaMemcpy(p->d_gates, hg.data(), hg.size() * sizeof(AdjGate), cudaMemcpyHostToDevice) != cudaSuccess) ||
      cudaMemset(p->d_flag, 0, sizeof(int)) != cudaSuccess) {
    qsv_adjoint_plan_destroy(p);
    return set_error(nullptr, QSV_ERR_CUDA, "plan tables: upload failed");
  }
  static bool configured = false;
  if (!configured) {
    cudaFuncSetAttribute(k_adj_corr_d<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, CORRD_SMEM);
    cudaFuncSetAttribute(k_adj_corr_d<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, CORRD_SMEM);
    cudaFuncSetAttribute(k_adj_corr_d<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, CORRD_SMEM);
    cudaFuncSetAttribute(k_adj_corr_d<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, CORRD_SMEM);
    cudaFuncSetAttribute(k_adj_walk, cudaFuncAttributeMaxDynamicSharedMemorySize, AT * AT * (int)sizeof(double2));
    configured = true;
  }
  *out = p;
  return QSV_OK;
}

extern "C" int qsv_adjoint_plan_destroy(qsv_adjoint_plan* p) {
  if (!p) return QSV_OK;
  for (FusedGeom* g : p->geom) fused_geom_destroy(g);
  if (p->d_blocks) cudaFree(p->d_blocks);
  if (p->d_gates) cudaFree(p->d_gates);
  if (p->d_flag) cudaFree(p->d_flag);
  delete p;
  return QSV_OK;
}

extern "C" size_t qsv_adjoint_scratch_bytes(const qsv_adjoint_plan* p, int nsets) {
  if (!p || nsets < 1) return 0;
  // Per set one W image, and per block and set one 128 x 128 FP64 correlation.
  return (size_t)nsets * (image_stride() + (size_t)p->nblocks * AKD * AKD * sizeof(double));
}

namespace {
int check_call(qsv_adjoint_plan* p, const void* psi, int nsets, const double* thetas, int nparams, void* scratch,
               size_t scratch_bytes) {
  if (!p) return set_error(nullptr, QSV_ERR_INVALID, "null plan");
  if (!psi || !thetas || nsets < 1) return set_error(nullptr, QSV_ERR_INVALID, "null state or angles, or no sets");
  if (nparams <= p->max_param) return set_error(nullptr, QSV_ERR_INVALID, "nparams smaller than the plan's parameters");
  if (!scratch || scratch_bytes < qsv_adjoint_scratch_bytes(p, nsets))
    return set_error(nullptr, QSV_ERR_INVALID, "scratch smaller than qsv_adjoint_scratch_bytes");
  if (((uintptr_t)scratch & 255) || ((uintptr_t)psi & 255))
    return set_error(nullptr, QSV_ERR_INVALID, "state and scratch must be 256-byte aligned");
  return QSV_OK;
}

int apply_block(qsv_adjoint_plan* p, int b, bool dagger, float2* const* states, int nstates, int nsets,
                const double* thetas, int nparams, uint8_t* images, cudaStream_t st) {
  const AdjBlockDev* blk = p->d_blocks + b;
  if (dagger)
    k_adj_images<true><<<nsets, A_THREADS, 0, st>>>(blk, p->d_gates, thetas, nparams, images, image_stride());
  else
    k_adj_images<false><<<nsets, A_THREADS, 0, st>>>(blk, p->d_gates, thetas, nparams, images, image_stride());
  int rc = check_stream_launch("adjoint images");
  if (rc) return rc;
  for (int i = 0; i < nstates; ++i) {
    rc = fused_geom_launch_sets(p->geom[(size_t)b], states[i], nsets, p->n, images, image_stride(), p->d_flag, st,
                                p->sm_count);
    if (rc) return set_error(nullptr, rc, "adjoint block launch failed");
  }
  return QSV_OK;
}
}  // namespace

extern "C" int qsv_adjoint_forward(qsv_adjoint_plan* p, void* psi, int nsets, const double* thetas, int nparams,
                                   void* scratch, size_t scratch_bytes, void* stream) {
  int rc = check_call(p, psi, nsets, thetas, nparams, scratch, scratch_bytes);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  float2* states[1] = {static_cast<float2*>(psi)};
  for (int b = 0; b < p->nblocks; ++b) {
    rc = apply_block(p, b, false, states, 1, nsets, thetas, nparams, static_cast<uint8_t*>(scratch), st);
    if (rc) return rc;
  }
  return QSV_OK;
}

extern "C" int qsv_adjoint_backward(qsv_adjoint_plan* p, void* psi, void* lam, int nsets, const double* thetas,
                                    int nparams, double* grads, int grad_stride, void* scratch,
                                    size_t scratch_bytes, void* stream) {
  int rc = check_call(p, psi, nsets, thetas, nparams, scratch, scratch_bytes);
  if (rc) return rc;
  if (!lam || !grads || grad_stride <= p->max_param || ((uintptr_t)lam & 255))
    return set_error(nullptr, QSV_ERR_INVALID, "bad lambda or gradient buffer");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  uint8_t* images = static_cast<uint8_t*>(scratch);
  // Correlations: one [nsets][128][128] slice per block, all walked in one launch at the end.
  double* corr_all = reinterpret_cast<double*>(images + (size_t)nsets * image_stride());
  const size_t slice = (size_t)nsets * AKD * AKD;
  QSV_CUDA(nullptr, cudaMemsetAsync(corr_all, 0, (size_t)p->nblocks * slice * sizeof(double), st));
  float2* states[2] = {static_cast<float2*>(psi), static_cast<float2*>(lam)};
  CorrArgs ca{};
  ca.psi = states[0];
  ca.lam = states[1];
  ca.tile_shift = p->n - 12;
  ca.ntiles = (uint64_t)nsets << ca.tile_shift;
  ca.n = p->n;
  ca.set_amps = 1ull << p->n;
  ca.flag = p->d_flag;
  auto grid_of = [&](const void* fn, int smem) -> unsigned {
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, CORR_THREADS, smem);
    per_sm = std::max(1, std::min(per_sm, 2));  // 256 TMEM columns each
    uint64_t grid = (uint64_t)std::max(1, p->sm_count) * per_sm;
    return (unsigned)std::min<uint64_t>(grid, ca.ntiles);
  };
  const unsigned grid_direct = grid_of((const void*)k_adj_corr_d<0>, CORRD_SMEM);
  for (int b = p->nblocks - 1; b >= 0; --b) {
    ca.blk = p->d_blocks + b;
    double* corr = corr_all + (size_t)b * slice;
    ca.corr = corr;
    if (fused_geom_backward_ok(p->geom[(size_t)b])) {
      // One pass: U^+ images, then un-compute and correlation together.
      k_adj_images<true><<<nsets, A_THREADS, 0, st>>>(p->d_blocks + b, p->d_gates, thetas, nparams, images,
                                                     image_stride());
      rc = check_stream_launch("adjoint images");
      if (rc) return rc;
      rc = fused_geom_launch_backward(p->geom[(size_t)b], states[0], states[1], corr, nsets, p->n, images,
                                      image_stride(), p->d_flag, st, p->sm_count);
      if (rc) return set_error(nullptr, rc, "adjoint backward launch failed");
      continue;
    }
    switch (p->corr_kind[(size_t)b]) {
      case 0: k_adj_corr_d<0><<<grid_direct, CORR_THREADS, CORRD_SMEM, st>>>(ca); break;
      case 1: k_adj_corr_d<1><<<grid_direct, CORR_THREADS, CORRD_SMEM, st>>>(ca); break;
      case 2: k_adj_corr_d<2><<<grid_direct, CORR_THREADS, CORRD_SMEM, st>>>(ca); break;
      default: k_adj_corr_d<3><<<grid_direct, CORR_THREADS, CORRD_SMEM, st>>>(ca); break;
    }
    rc = check_stream_launch("adjoint correlation");
    if (rc) return rc;
    rc = apply_block(p, b, true, states, 2, nsets, thetas, nparams, images, st);
    if (rc) return rc;
  }
  // Every block's gradients from its correlation, in one launch.
  k_adj_walk<<<dim3((unsigned)nsets, (unsigned)p->nblocks), A_THREADS, AT * AT * sizeof(double2), st>>>(
      p->d_blocks, p->d_gates, thetas, nparams, corr_all, grads, grad_stride);
  return check_stream_launch("adjoint walk");
}

extern "C" int qsv_adjoint_plan_fused_blocks(const qsv_adjoint_plan* p, int* out) {
  if (!p || !out) return set_error(nullptr, QSV_ERR_INVALID, "null plan or output");
  int count = 0;
  for (FusedGeom* g : p->geom) count += fused_geom_backward_ok(g) ? 1 : 0;
  *out = count;
  return QSV_OK;
}

extern "C" int qsv_adjoint_status(qsv_adjoint_plan* p) {
  if (!p) return set_error(nullptr, QSV_ERR_INVALID, "null plan");
  int flag = 0;
  QSV_CUDA(nullptr, cudaMemcpy(&flag, p->d_flag, sizeof(int), cudaMemcpyDeviceToHost));
  if (flag) {
    cudaMemset(p->d_flag, 0, sizeof(int));
    return set_error(nullptr, QSV_ERR_TIMEOUT, "a bounded device wait of the adjoint gave up (code %d)", flag);
  }
  return QSV_OK;
}

namespace qsv {
int oob_take_adjtc(unsigned long long* count, unsigned long long* first) {
#ifdef QSV_BOUNDS_CHECK
  return qsv_oob_take_unit(count, first);
#else
  (void)count;
  (void)first;
  return 0;
#endif
}
}  // namespace qsv
