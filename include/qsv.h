/*
 * qsv.h — C ABI of the GB300 state-vector library (libqsv.so).
 *
 * The library holds one dense 2^n state vector per handle in HBM (complex64 or
 * complex128, interleaved re/im, amplitude index bit (n-1-q) holds qubit q, so qubit 0
 * is the most significant bit — the reference's convention, qip/ext/kronprod.pyx:168).
 * Every call is asynchronous on the handle's CUDA stream unless it returns a host
 * value.  Every entry point returns an int status (QSV_OK == 0); qsv_last_error()
 * gives the message of the last failure on a handle.  No entry point traps, asserts on
 * the device or spins without a bound: device-side waits give up with QSV_ERR_TIMEOUT.
 *
 * Qubit indices in every call use the reference's global qubit index (0 = MSB).
 * A matrix acting on targets (t_0, ..., t_{k-1}) is 2^k x 2^k complex128, row-major,
 * interleaved, with t_0 the most significant bit of the row/column index
 * (qip/ext/kronprod.pyx:184-189).
 *
 * Each declaration names the reference interface it replaces (path within the
 * Renmusxd/QIP project).
 */
#ifndef QSV_H
#define QSV_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct qsv_state qsv_state;

enum qsv_dtype { QSV_C64 = 0, QSV_C128 = 1 };

enum qsv_status {
  QSV_OK = 0,
  QSV_ERR_INVALID = 1,     /* bad argument: maps to ValueError / Exception          */
  QSV_ERR_OOM = 2,         /* device allocation failed: maps to MemoryError         */
  QSV_ERR_CUDA = 3,        /* a CUDA runtime call failed                             */
  QSV_ERR_TIMEOUT = 4,     /* a bounded device wait gave up                          */
  QSV_ERR_UNSUPPORTED = 5  /* valid request outside what the library implements      */
};

/* ---- lifetime --------------------------------------------------------------------
 * Replaces the numpy state/arena pair that CythonBackend owns
 * (qip/backend.py:68-71, 88, 103).  One device buffer; updates are in place, so there
 * is no arena.  The state starts as |0...0>. */
int qsv_create(int n, int dtype, qsv_state** out);
/* Fault injection for tests: with QSV_INJECT_ALLOC_FAILURE set (not "0") qsv_create
 * fails with QSV_ERR_OOM before any device call. */
/* qsv_destroy parks the buffers of a healthy state (at most two states' worth; amplitude
 * buffers up to 8 GiB in total) and the next qsv_create on that device reuses
 * them (the amplitude buffer when the size matches), so a create / run / read / destroy
 * loop allocates nothing after its first state.  A failed allocation in qsv_create
 * releases the parked buffers and retries; qsv_trim releases them on request. */
int qsv_destroy(qsv_state* s);
int qsv_trim(void);
/* Bounds-checked build (libqsv_checked.so, compiled with -DQSV_BOUNDS_CHECK): every
 * kernel tests each computed state index against the state's size before the access,
 * counts bad ones and skips them (nothing traps).  qsv_bounds_report waits for the
 * device, returns the count and the first bad index since the last report, and clears
 * them.  In the normal build it returns QSV_ERR_UNSUPPORTED.  No reference counterpart
 * (the reference compiles its kernels without bounds checks, kronprod.pyx:41-42). */
int qsv_bounds_report(unsigned long long* count, unsigned long long* first_index);
/* Use an external CUDA stream (cudaStream_t passed as void*; NULL = the handle's own). */
int qsv_set_stream(qsv_state* s, void* stream);
int qsv_synchronize(qsv_state* s);
int qsv_num_qubits(const qsv_state* s);
int qsv_dtype(const qsv_state* s);
/* Device pointer of the amplitude buffer (for zero-copy interop). */
void* qsv_device_ptr(qsv_state* s);
const char* qsv_last_error(const qsv_state* s);
const char* qsv_status_string(int status);
/* Number of kernels this library launched in the calling process so far. */
unsigned long long qsv_launch_count(void);

/* ---- state preparation / readout -------------------------------------------------- */
/* Product state from fed registers.  Replaces CythonBackend.make_state and
 * qip.util.gen_edit_indices (qip/backend.py:73-104, qip/util.py:108-124):
 * amp[i] = prod_g feed_g[bits of i at group g's qubits, first qubit = MSB] when every
 * unfed qubit of i is 0, else 0; no feeds -> |0...0>.  Feeds are complex128,
 * concatenated in group order (group g holds 2^group_sizes[g] values); not normalised. */
int qsv_set_product_state(qsv_state* s, int ngroups, const int* group_sizes,
                          const int* qubits_flat, const double* feeds_c128);
/* Overwrite amplitudes [start, start+count) from host data of the handle's dtype.
 * Replaces StateType.overwrite_relative_range (qip/backend.py:171-172). */
int qsv_write_range(qsv_state* s, const void* host, uint64_t start, uint64_t count);
/* Add host data to amplitudes [start, start+count).
 * Replaces StateType.addto_relative_range (qip/backend.py:174-175). */
int qsv_add_range(qsv_state* s, const void* host, uint64_t start, uint64_t count);
/* Copy amplitudes [start, start+count) to host memory of the handle's dtype.  Blocks.
 * Replaces CythonBackend.get_state / get_relative_range (qip/backend.py:106-107,168-169). */
int qsv_read_range(qsv_state* s, void* host, uint64_t start, uint64_t count);
/* NVTX ranges (a profiler shows them on its timeline; no-ops otherwise).  No reference
 * counterpart: the graph executor opens one per node when QSV_NVTX=1. */
int qsv_trace_push(const char* name);
int qsv_trace_pop(void);
/* Page-locked host buffers (cudaHostAlloc / cudaFreeHost).  A read into one is a
 * single DMA with no staging copy and no page faults.  No reference counterpart: the
 * reference's state already lives in host memory. */
int qsv_host_alloc(uint64_t bytes, void** out);
int qsv_host_free(void* p);

/* ---- gates (kronselect_dot) ---------------------------------------------------------
 * The reference applies every gate through cdot_loop (qip/ext/kronprod.pyx:41-200) via
 * StateType.kronselect_dot (qip/backend.py:112-116).  The host layer splits a
 * kronselect_dot dict into the calls below; each is in place.  Controls must all be 1
 * (the CMat structure, qip/operators.py:233-268, kronprod.pyx:215-225). */

/* Dense 2^k x 2^k matrix on k targets (1 <= k <= 5), optional controls. */
int qsv_apply_matrix(qsv_state* s, int k, const int* targets, int ncontrols,
                     const int* controls, const double* mat_c128);
/* Diagonal matrix diag(d_0..d_{2^k-1}) on k targets (k <= 10), optional controls.
 * Only amplitudes whose diagonal entry differs from 1 are read or written. */
int qsv_apply_diagonal(qsv_state* s, int k, const int* targets, int ncontrols,
                       const int* controls, const double* diag_c128);
/* Monomial matrix (exactly one non-zero per row): out[r] = phase[r] * in[perm[r]].
 * Entries whose phase is exactly 1 move data without arithmetic (bit-exact). */
int qsv_apply_monomial(qsv_state* s, int k, const int* targets, int ncontrols,
                       const int* controls, const int* perm, const double* phase_c128);
/* Exchange the m-qubit register a with register b (SwapMat, qip/operators.py:157-179,
 * kronprod.pyx:227-231), optional controls.  Pure data movement, bit-exact. */
int qsv_apply_swap(qsv_state* s, int m, const int* a, const int* b, int ncontrols,
                   const int* controls);
/* Fused dense blocks on the tensor cores (complex64 handles only): for each block b,
 * a 2^k_b x 2^k_b matrix (4 <= k_b <= 6) applied to all 2^(n-k_b) groups as a
 * split-bf16 GEMM with FP32 accumulation (tcgen05).  No reference counterpart: the
 * reference applies one kronselect_dot dict per pass (kronprod.pyx:157). */
int qsv_apply_blocks(qsv_state* s, int nblocks, const int* ks, const int* targets_flat,
                     const double* mats_c128);

/* Device-resident fused-block plan: the block images are built and uploaded once, so
 * qsv_plan_launch issues kernels only (no host work, no copies) and can be captured in
 * a CUDA graph.  Same semantics as qsv_apply_blocks.  No reference counterpart. */
typedef struct qsv_plan qsv_plan;
int qsv_plan_create(qsv_state* s, int nblocks, const int* ks, const int* targets_flat,
                    const double* mats_c128, qsv_plan** out);
int qsv_plan_launch(qsv_state* s, const qsv_plan* p, int first, int count);
int qsv_plan_destroy(qsv_plan* p);
/* Fault injection for tests of the bounded device waits (no reference counterpart: the
 * reference's failure handling is host-side, qip/distributed/manager.py:219-236).  Arms
 * the next fused-block launch on this handle (qsv_apply_blocks or qsv_plan_launch):
 * in every CTA, the first wait for a tile's products waits on an mbarrier that nothing
 * arrives on and gives up after wait_ns (1 us .. 1 s).  The kernel then waits (bounded,
 * 2 s) for the products it has in flight, frees its tensor memory, sets the handle's
 * status word and returns; it stores nothing, so the state is unchanged.  The next
 * qsv_synchronize returns QSV_ERR_TIMEOUT and clears the status word; the handle stays
 * usable. */
int qsv_inject_block_stall(qsv_state* s, uint64_t wait_ns);

/* Fusion planning on the host (no reference counterpart).  Gates are given as qubit bit
 * masks (bit q <-> qubit q) and amp-update weights.  Each round grows up to lookahead
 * candidate blocks (candidate s leaves the first s pending gates out, then takes every
 * later gate whose qubits fit in kmax and are not blocked by a gate left out before it;
 * a left-out gate blocks its qubits) and keeps the one with the best score: its weight
 * plus (lookahead2 > 0) the most weight one of the next round's first lookahead2
 * candidates would take after it.  A gate wider than kmax at the front is its own step.  nqubits < 0: plan every gate.
 * nqubits >= 0 (prefix mode): stop at the first round later gates could change (a
 * candidate is final once it holds min(kmax, nqubits) qubits, all blocked; strict: all
 * candidates of both levels must be final, else the best one), except that a round is decided on the
 * pending gates anyway while more than min_pending (> 0) are pending: the block is just
 * as valid, it may only be smaller than later gates would have allowed.
 * beam_width or beam_branch > 1: a beam search over rounds replaces the rounds where the
 * whole list is planned (nqubits < 0) and, in prefix mode, for the steps taken while
 * more than min_pending gates are pending.  Each kept state (a list of unplanned gates)
 * offers its beam_branch best distinct candidates (most weight first; ties: earlier
 * start); of all children (merged when they planned the same gate set) the beam_width
 * with the least weight left go on.  Output: the planned gates in step
 * order (order_out, ngates entries of room), step s = order_out[step_start_out[s] ..
 * step_start_out[s+1]) (ngates + 1 entries of room), nsteps, number of planned gates. */
int qsv_fusion_plan(int ngates, const uint64_t* qmask, const double* weight, int kmax,
                    int lookahead, int lookahead2, int beam_width, int beam_branch, int nqubits,
                    int strict, int min_pending, int* order_out, int* step_start_out,
                    int* nsteps_out, int* nplanned_out);
/* Dense matrices of fused blocks (host, threads across blocks; no reference
 * counterpart).  Block b has block_k[b] qubits (block_qubits, ascending: the first is
 * the MSB of the block index) and block_ngates[b] gates; gate g acts on gate_nq[g]
 * qubits (gate_qubits, its first the MSB of its index) with the row-major complex
 * matrix gate_mats (2^q x 2^q, interleaved re/im).  out: block b's 2^k x 2^k complex
 * matrix = product of its gates in order (later gates on the left). */
int qsv_block_matrices(int nblocks, const int* block_k, const int* block_qubits,
                       const int* block_ngates, const int* gate_nq, const int* gate_qubits,
                       const double* gate_mats, double* out);

/* Access-mode autotuning of the tensor-core block kernel.  No reference counterpart
 * (the reference has no GPU path).  A placement class is (k, low_mask): bit p of
 * low_mask set <-> a target on address bit p, p < 7 (targets on higher bits do not
 * change how a tile is read).  Modes: 0 direct, 1 staged (shared-memory transpose),
 * 2 shuffle (warp exchanges; needs 1..k-1 targets on bits 0..4), 3 prefix (transposed
 * products; k = 6 with targets on bits 0, 1 and 2), 4 pair1 / 5 pair2 (transposed
 * products; k = 6 with the lowest target on bit 1 / bit 2).  Without a
 * recorded choice a class
 * takes the built-in rule: direct when its low targets are bits 0..L-1 with L <= 3,
 * prefix for k = 6 with L >= 4, pair1 / pair2 when the lowest target is on bit 1 / 2
 * and at least 3 of bits 1..4 / 2..5 are targets, direct when no target sits on bits
 * 0..2, else shuffle (or staged).  Choices are kept per device
 * for the life of the process and used by qsv_apply_blocks / qsv_plan_create and the
 * tensor-core adjoint.
 *
 * qsv_tune_blocks times every applicable mode of each class (reps launches after one
 * warm-up) on a zeroed scratch state of min(n, 26) qubits (the caller's state is not
 * touched), writes out_ms[6*i + mode] (-1 where a mode does not apply) and out_mode[i],
 * and records the fastest.  Synchronises the handle's stream.
 * qsv_set_block_mode pins a mode for a class (mode -1 restores the built-in rule). */
int qsv_tune_blocks(qsv_state* s, int count, const int* ks, const int* low_masks, int reps,
                    double* out_ms, int* out_mode);
int qsv_set_block_mode(qsv_state* s, int k, int low_mask, int mode);

/* ---- measurement ---------------------------------------------------------------------
 * Marginal probabilities over m qubits, FP64 compensated sums, out[2^m].
 * Outcome bit j <-> qubits[j] (LSB first), as measure_probabilities
 * (qip/ext/kronprod.pyx:238-261).  m = 0 gives the squared norm (prob_magnitude,
 * kronprod.pyx:318-326). */
int qsv_probabilities(qsv_state* s, int m, const int* qubits, double* out);
/* Squared norm sum |amp|^2 (FP64).  Replaces prob_magnitude / StateType.total_prob
 * (kronprod.pyx:318-326, qip/backend.py:123-124). */
int qsv_norm2(qsv_state* s, double* out);
/* Single-qubit marginals P(q = 1) of every qubit in one pass, out[n], plus the squared
 * norm in *norm2.  No reference counterpart (one StochasticMeasure per qubit there). */
int qsv_qubit_marginals(qsv_state* s, double* out, double* norm2);
/* Collapse onto the outcome where the m measured qubits equal `value` (bit j of value
 * <-> qubits[j], LSB first) and scale the kept amplitudes by `scale` (FP64).
 * Replaces the collapse loop of measure (kronprod.pyx:430-444). */
int qsv_collapse(qsv_state* s, int m, const int* qubits, uint64_t value, double scale);
/* Collapse and remove the measured qubits: the state shrinks to 2^(n-m) amplitudes,
 * remaining qubits keep their order.  Replaces reduce_measure (kronprod.pyx:449-490). */
int qsv_reduce(qsv_state* s, int m, const int* qubits, uint64_t value, double scale);

/* Marginal probabilities of a caller-owned state without allocating device memory.
 * No counterpart in the reference.  For callers that cannot call cudaMalloc when they
 * need the distribution — their device memory belongs to another allocator (e.g. a
 * framework that has reserved all of HBM), or they run in a loop where allocating is
 * not allowed.  Same result as qsv_probabilities (out[v], bit j of v <-> qubits[j]) for
 * a state of 2^n amplitudes of `dtype` at device address d_amp; d_out is a device
 * buffer of 2^m doubles; work is queued on `stream` (NULL = the default stream) and
 * nothing is copied to the host.  Partial sums use a file-scope device array of 2^16
 * doubles (512 KiB, held by every GPU that loads the library until exit), so
 * m <= QSV_STATIC_MAX_MEASURED (16); larger m returns QSV_ERR_INVALID.  The first call
 * on a device looks up that array's address (once per device, with the device
 * current), so make the first call before any stream capture.  Every call shares the
 * array: calls that overlap on the GPU (different streams, or concurrent threads)
 * race and must be ordered by the caller.  Errors: qsv_last_error(NULL). */
#define QSV_STATIC_MAX_MEASURED 16
int qsv_probabilities_static(const void* d_amp, int n, int dtype, int m, const int* qubits,
                             double* d_out, void* stream);

/* <a|b> = sum conj(a_i) b_i in FP64 (compensated), states of equal n, any dtypes.
 * Used for infidelity 1 - |<a|b>|^2 / (<a|a><b|b>).  No reference counterpart. */
int qsv_inner_product(qsv_state* a, qsv_state* b, double* re, double* im);

/* ---- batched states and adjoint gradients ----------------------------------------------
 * A batch is nsets states of 2^n amplitudes back to back in one caller-owned device
 * buffer (e.g. a [nsets, 2^n] torch tensor); every call is asynchronous on `stream`.
 * No reference counterpart: the reference has no batching and no gradients; these serve
 * the adjoint-method differentiation of parameterised circuits. */
/* Every state of the batch := |0...0>. */
int qsv_batch_reset(void* psi, int nsets, int n, int dtype, void* stream);
/* Per-gate, per-set 2x2 matrices of a rotation circuit, built on the device: gate g has
 * kind_param[2g] = 0 (RY(theta) = exp(-i theta Y/2)), 1 (RZ(theta) = exp(-i theta Z/2)) or
 * 2 (CNOT: X on its target) and kind_param[2g+1] = its parameter index; theta of set s is
 * thetas[s * nparams + parameter] (device doubles).  U[(g * nsets + s) * 4 ..] row-major in
 * the batch's dtype, Ud = U^+ likewise (all device memory). */
int qsv_batch_rotation_matrices(const double* thetas, int nsets, int nparams, int ngates,
                                const int* kind_param, int dtype, void* U, void* Ud, void* stream);
/* psi[s] <- M_s psi[s] on `target` (qubit index), controlled by `control` (-1: none);
 * mats holds nsets row-major 2x2 matrices of the batch's dtype. */
int qsv_batch_apply_1q(void* psi, int nsets, int n, int dtype, int target, int control,
                       const void* mats, void* stream);
/* lambda[s] := (sum_i Z_i) psi[s] and energies[s] := <psi[s]| sum_i Z_i |psi[s]> (FP64,
 * device array).  scratch: caller-owned device doubles for partial sums. */
int qsv_batch_observable_sumz(const void* psi, void* lam, int nsets, int n, int dtype,
                              double* energies, double* scratch, size_t scratch_doubles,
                              void* stream);
/* One adjoint step for gate g: when generator is 1 (Y) or 2 (Z) the gate is
 * exp(-i theta P/2) on `target` and grads[s * grad_stride] := Im <lambda[s]| P |psi[s]>
 * (= dE/dtheta); then psi[s] <- M_s psi[s] and lambda[s] <- M_s lambda[s] with
 * M_s = U_s^+ given in mats_dagger. */
int qsv_batch_adjoint_step(void* psi, void* lam, int nsets, int n, int dtype, int target,
                           int control, const void* mats_dagger, int generator, double* grads,
                           int grad_stride, double* scratch, size_t scratch_doubles,
                           void* stream);

/* Segmented batch execution (cache blocking; no reference counterpart).  A segment is a
 * run of single-qubit gates (optionally controlled) whose qubits lie in lb local bit
 * positions lpos[0..lb) (ascending; complex64 lb <= 13, complex128 lb <= 12).  For every
 * chunk of 2^lb amplitudes (fixed values of the other bits) of every set the chunk is
 * brought into shared memory once and all the segment's gates are applied there.
 * Gates come in groups of at most 3 local bits and 8 gates, each applied in registers
 * to items of 2^nb amplitudes (one shared-memory pass per group).
 * groups_dev: device array of ngroups records {int32 nb (1..3), int32 local bit
 * positions packed 8 bits each (ascending), int32 first gate, int32 gate count}.
 * gates_dev: device array of ngates records {int32 target index among its group's bits,
 * int32 control index or -1, int32 gate index g, int32 (generator << 24) | parameter};
 * the 2x2 matrix of gate g for set s is at mats[(g * nsets + s) * 4], row-major, the
 * state's dtype.  At most 512 gates and 256 generator gates per segment.
 * forward: psi <- (gates in order) psi.
 * adjoint: groups and their gates in reverse order: generator 1 (Y) / 2 (Z):
 * grads[s * grad_stride + parameter] += Im <lambda| P |psi>; then psi, lambda <- M psi,
 * M lambda with M the supplied matrix (U^+).  grads accumulate (FP64 atomics), so zero
 * them first. */
int qsv_batch_segment_forward(void* psi, int nsets, int n, int dtype, int lb, const int* lpos,
                              int ngroups, const void* groups_dev, int ngates, const void* gates_dev,
                              const void* mats, void* stream);
int qsv_batch_segment_adjoint(void* psi, void* lam, int nsets, int n, int dtype, int lb,
                              const int* lpos, int ngroups, const void* groups_dev, int ngates,
                              const void* gates_dev, const void* mats_dagger, double* grads,
                              int grad_stride, void* stream);

/* ---- adjoint gradients on the tensor cores ---------------------------------------------
 * No reference counterpart (the reference has no gradients).  For complex64 batches of
 * nsets states (13 <= n <= 34) of a circuit of rotations RY(theta) = exp(-i theta Y/2),
 * RZ(theta) = exp(-i theta Z/2) and CNOTs, split by the caller into blocks of six qubits
 * (a valid execution order of the circuit, e.g. the fusion planner's).
 * block_qubits: 6 ascending qubit indices per block; block_ngates[b]: gates of block b;
 * gates: 4 ints per gate, blocks one after another, each block's gates in execution
 * order: kind (0 RY, 1 RZ, 2 CNOT), target qubit, control qubit (CNOT; else -1),
 * parameter index (rotations; else -1).  The plan uploads its tables once.
 * qsv_adjoint_forward: psi[s] <- U_blocks psi[s], each set's block matrices built on the
 * device from its angles thetas[s * nparams + p] (device doubles) and applied as
 * split-bf16 tensor-core products (as qsv_apply_blocks).
 * qsv_adjoint_backward: psi = the final states, lam = H psi; for the blocks in reverse,
 * one tensor-core correlation X = sum_g psi[g] lam[g]^+ over the other qubits gives every
 * gradient of the block (dE/dtheta_j = Im Tr(P_j Q_j), Q walked through the block's gates
 * in FP64), added to grads[s * grad_stride + p]; then psi, lam <- U^+ psi, U^+ lam.  For
 * blocks in the direct, prefix and pair access modes the correlation and both un-computes
 * are one pass over psi and lam; qsv_adjoint_plan_fused_blocks writes how many blocks of
 * the plan take it to *out (the others use three passes).
 * scratch: caller-owned device memory of qsv_adjoint_scratch_bytes (per set one block
 * image, and per block and set one 128 x 128 FP64 correlation, all walked to gradients in
 * one launch at the end of the backward; nblocks <= 65535); psi, lam and scratch
 * 256-byte aligned; work queued on `stream`.
 * qsv_adjoint_status synchronises and reports a bounded device wait that gave up
 * (QSV_ERR_TIMEOUT).  Errors: qsv_last_error(NULL). */
typedef struct qsv_adjoint_plan qsv_adjoint_plan;
int qsv_adjoint_plan_create(int n, int nblocks, const int* block_qubits, const int* block_ngates,
                            const int* gates, qsv_adjoint_plan** out);
int qsv_adjoint_plan_destroy(qsv_adjoint_plan* p);
size_t qsv_adjoint_scratch_bytes(const qsv_adjoint_plan* p, int nsets);
int qsv_adjoint_plan_fused_blocks(const qsv_adjoint_plan* p, int* out);
int qsv_adjoint_forward(qsv_adjoint_plan* p, void* psi, int nsets, const double* thetas, int nparams,
                        void* scratch, size_t scratch_bytes, void* stream);
int qsv_adjoint_backward(qsv_adjoint_plan* p, void* psi, void* lam, int nsets, const double* thetas,
                         int nparams, double* grads, int grad_stride, void* scratch,
                         size_t scratch_bytes, void* stream);
int qsv_adjoint_status(qsv_adjoint_plan* p);

/* ---- many small circuits in one persistent launch --------------------------------------
 * No reference counterpart (the reference runs one circuit per run() call).  A batch
 * object holds a gate table, a circuit table, per-qubit product-state feeds and the
 * output states of every circuit in device memory.  qsv_circuits_run replays one
 * persistent launch (captured once into a CUDA graph on the given, non-default
 * stream), in clusters of CS CTAs (one CTA per SM; CS = 6, QSV_CIRCUIT_CLUSTER = 1..8
 * overrides).  The leading circuits of the table with n >= 14 + log2(2 CS) run one per
 * cluster (the cluster's CTAs share each segment's chunks), the rest one per CTA, each
 * group taken in table order from its own atomic counter (so put the largest streamed
 * circuits first, then the rest longest first); n <= 14 circuits run entirely in shared
 * memory. */
typedef struct qsv_circuits qsv_circuits;
/* Gate record (48 bytes).  kind 0 DENSE1: 2x2 complex64 m on q0; 1 PHASE1: |1> of q0 gets
 * phase (m[0], m[1]); 2 X on q0; 3 CX: target q0, control q1; 4 CSWAP: control q0, swap
 * q1 and q2.  Qubit indices: 0 = most significant bit of the circuit's state. */
struct qsv_gate_rec {
  int32_t kind;
  int32_t q0, q1, q2;
  float m[8];
};
/* Circuit record (32 bytes): n (3..24), gate count, offset of its first gate, offset of
 * its output state (amplitudes) and of its feeds (2 complex64 values per qubit, qubit 0
 * first; the input is the product of the per-qubit feeds). */
struct qsv_circuit_rec {
  int32_t n, ngates;
  int64_t gate_offset;
  int64_t state_offset;
  int64_t feed_offset;
};
int qsv_circuits_create(const void* gates, int64_t ngates, const void* circuits, int ncircuits,
                        const void* feeds_c64, int64_t nfeeds, qsv_circuits** out);
int qsv_circuits_run(qsv_circuits* b, void* stream);
/* Final state of one circuit (2^n complex64) to host memory.  Blocks. */
int qsv_circuits_read(qsv_circuits* b, int circuit, void* host_out);
/* Per-circuit device timestamps [start, end] in ns (2 * ncircuits values).  Blocks. */
int qsv_circuits_times(qsv_circuits* b, unsigned long long* host_out);
int qsv_circuits_destroy(qsv_circuits* b);

/* ---- function oracle -----------------------------------------------------------------
 * |x>|q>|r> -> |x>|f(x) xor q>|r> with f given as a table of 2^n1 values.
 * Replaces func_apply (qip/ext/func_apply.pyx:9-112). */
int qsv_func_apply(qsv_state* s, int n1, const int* reg1, int n2, const int* reg2,
                   const int64_t* table);

#ifdef __cplusplus
}
#endif

#endif /* QSV_H */
