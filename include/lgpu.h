/*
 * lgpu.h — the C ABI of the GB300 statevector engine (liblgpu_gb300.so).
 *
 * Every entry point is plain C: device pointers, sizes, host arrays and a
 * CUDA stream.  No C++ or torch types cross this boundary.  The C++ drop-in
 * classes (StateVectorCudaManaged<T>, AdjointJacobianGPU<T>, the observable
 * family) are the intended callers; they replace the closed-library calls of
 * the reference PennyLane-Lightning-GPU 0.33 at the file:line cited beside
 * each function.
 *
 * Conventions
 *   - A state is 2^n contiguous amplitudes, interleaved (re, im):
 *     LGPU_C64 = float2 (8 B), LGPU_C128 = double2 (16 B).
 *   - Qubits are addressed by STATE-INDEX BIT positions (0 = least
 *     significant).  PennyLane wire w of an n-qubit state is bit n-1-w; the
 *     C++ layer performs that mapping.
 *   - Matrices are row-major 2^t x 2^t complex128 (interleaved doubles);
 *     matrix row/column index bit (t-1-k) corresponds to tgts[k] (the first
 *     target is the most significant matrix bit).
 *   - Controls: bits that must equal ctrl_vals[k] (NULL = all ones).
 *   - Results of reductions are written to `out`; when out_on_device is 0
 *     the call synchronises the stream and `out` is host memory, otherwise
 *     `out` is device memory and the call is asynchronous.
 *   - The library never frees caller memory.  Scratch memory for reductions
 *     and sampling comes from an lgpu_context_t owned by the caller; a context
 *     must not be used from two streams at the same time.
 *   - Every function returns an lgpu_status_t; lgpu_last_error_string()
 *     holds the message of the last failure on the calling thread.
 */
#ifndef LGPU_H
#define LGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *lgpu_stream_t; /* identical to cudaStream_t */

typedef enum {
    LGPU_OK = 0,
    LGPU_ERR_INVALID_ARG = 1,
    LGPU_ERR_OOM = 2,
    LGPU_ERR_CUDA = 3,
    LGPU_ERR_TIMEOUT = 4,
    LGPU_ERR_UNSUPPORTED = 5,
    LGPU_ERR_NO_DEVICE = 6
} lgpu_status_t;

typedef enum { LGPU_C64 = 0, LGPU_C128 = 1 } lgpu_dtype_t;

typedef enum { LGPU_H2D = 0, LGPU_D2H = 1, LGPU_D2D = 2 } lgpu_copy_kind_t;

#define LGPU_MAX_QUBITS 34
#define LGPU_MAX_DENSE_TARGETS 12
#define LGPU_MAX_EXPVAL_TARGETS 13
#define LGPU_MAX_CONTROLS 16

typedef struct lgpu_context_s *lgpu_context_t;

/* ---- library / errors ------------------------------------------------ */
/* Errors: the reference raises LightningException from PL_CUDA_IS_SUCCESS /
 * PL_CUSTATEVEC_IS_SUCCESS (cuda_helpers.hpp:48-80); here every call returns a
 * status and lgpu_last_error_string() holds the message (thread-local). */
int lgpu_abi_version(void);
const char *lgpu_last_error_string(void);

/* complex128 arithmetic mode of the streaming gate kernels (process-wide):
 * 0 = native FP64; 1 (default) = one FP64 FMA plus one integer-pipe multiply
 * per output component, which halves FP64 issue on GB300 (whose FP64 rate is
 * about 2 FMA/clock/SM).  The integer multiply equals the IEEE product except
 * on exact rounding ties.  The environment variable LGPU_F64_EMUL=0 selects
 * mode 0 at start-up.  No counterpart in the reference (cuStateVec chooses
 * its arithmetic internally). */
lgpu_status_t lgpu_set_f64_mode(int mode);
int lgpu_get_f64_mode(void);

/* Kernel family for uncontrolled 1-target gates on states of >= 13 (c128) /
 * 14 (c64) qubits (process-wide): 1 (default) = persistent CTAs streaming
 * 64 KB tiles through a 3-stage shared-memory ring with cp.async.bulk loads
 * and stores; 0 = grid-stride kernel.  LGPU_BULK=0 selects 0 at start-up.
 * No counterpart in the reference. */
lgpu_status_t lgpu_set_stream_mode(int mode);
int lgpu_get_stream_mode(void);

/* Kernel family for dense 6-target complex64 matrices on the six lowest state
 * bits (any target order, no controls, n >= 12) (process-wide): 1 (default) =
 * tensor cores (tcgen05.mma kind::tf32, three TF32 products per FP32 value,
 * FP32 accumulation in tensor memory); 0 = the shared-memory FP32 kernel used
 * for every other dense matrix of 6..12 targets.  LGPU_TC=0 selects 0 at
 * start-up.  No counterpart in the reference (custatevecApplyMatrix chooses
 * its kernels internally). */
lgpu_status_t lgpu_set_tensor_mode(int mode);
int lgpu_get_tensor_mode(void);

/* Device-side error flag of the engine's bounded waits (1 = a kernel gave up
 * waiting for a bulk copy and left its tile unprocessed).  reset != 0 clears
 * it.  The C++ layer checks it at every synchronisation point.  No
 * counterpart in the reference. */
lgpu_status_t lgpu_device_error(int *code, int reset);

/* The same per stream: 1 when a kernel launched on `stream` gave up waiting
 * since the last reset of this stream's word; reset != 0 clears it.  The
 * call synchronises `stream`.  The default streams share one word; other
 * streams get their own (beyond 255 distinct streams, words are shared
 * round-robin).  The C++ layer checks its own stream's word at every
 * synchronisation, so a time-out on one stream is not raised at another's.
 * No counterpart in the reference. */
lgpu_status_t lgpu_stream_error(lgpu_stream_t stream, int *code, int reset);

/* Diagnostic of the bounded waits: one CTA waits on an mbarrier that expects
 * bytes no copy will deliver, with the streaming kernels' give-up logic and a
 * limit of `spin_limit` polls (at most 2^24); the call synchronises `stream`
 * and leaves the time-out recorded for lgpu_device_error.  No counterpart in
 * the reference. */
lgpu_status_t lgpu_selftest_bounded_wait(uint32_t spin_limit, lgpu_stream_t stream);

/* ---- device and memory (DataBuffer.hpp:31-218; cuda_helpers.hpp:600-650,
 *      getGPUCount / getGPUIdx / deviceReset / getGPUArch; Bindings.cpp:1736-1748;
 *      the C++ layer needs no CUDA runtime of its own) */
lgpu_status_t lgpu_device_count(int *count);
lgpu_status_t lgpu_get_device(int *device);
lgpu_status_t lgpu_set_device(int device);
lgpu_status_t lgpu_device_arch(int device, int *major, int *minor);
lgpu_status_t lgpu_device_sm_count(int device, int *sms);
lgpu_status_t lgpu_device_reset(void);
lgpu_status_t lgpu_mem_info(size_t *free_bytes, size_t *total_bytes);
lgpu_status_t lgpu_malloc(void **ptr, size_t bytes);
lgpu_status_t lgpu_free(void *ptr);
/* Stream-ordered allocation from the device's memory pool, which keeps freed
 * blocks for reuse instead of returning them to the driver: neither call
 * synchronises the device (cudaFree does), so states created and destroyed on
 * different streams do not wait for each other's kernels.  The memory is
 * usable in stream order on `stream`; other streams must order themselves
 * after it.  No counterpart in the reference. */
lgpu_status_t lgpu_malloc_async(void **ptr, size_t bytes, lgpu_stream_t stream);
lgpu_status_t lgpu_free_async(void *ptr, lgpu_stream_t stream);
lgpu_status_t lgpu_host_alloc_pinned(void **ptr, size_t bytes);
lgpu_status_t lgpu_host_free_pinned(void *ptr);
lgpu_status_t lgpu_memcpy(void *dst, const void *src, size_t bytes, lgpu_copy_kind_t kind,
                          int async, lgpu_stream_t stream);
lgpu_status_t lgpu_memset(void *dst, int value, size_t bytes, lgpu_stream_t stream);
lgpu_status_t lgpu_stream_create(lgpu_stream_t *stream);
lgpu_status_t lgpu_stream_destroy(lgpu_stream_t stream);
lgpu_status_t lgpu_stream_sync(lgpu_stream_t stream);
lgpu_status_t lgpu_peer_access_all(void);

/* ---- scratch context ----------------------------------------------------
 * Replaces the per-state library handles and their workspaces: the
 * cuStateVec / cuBLAS / cuSPARSE handles of StateVectorCudaManaged
 * (StateVectorCudaManaged.hpp:83-134, the SharedCusvHandle / CublasCaller /
 * SharedCusparseHandle arguments), the per-call workspace queries and
 * cudaMalloc/cudaFree around custatevecApplyMatrix and
 * custatevecComputeExpectation (:1433-1471, :1602-1639), and CublasCaller's
 * mutex-guarded handle (cuda_helpers.hpp:433-440), all made by
 * make_shared_cublas_caller / make_shared_cusv_handle /
 * make_shared_cusparse_handle (cuda_helpers.hpp:817-839).  A context holds the
 * reduction scratch and pinned staging of one device. */
lgpu_status_t lgpu_context_create(int device, lgpu_context_t *ctx);
lgpu_status_t lgpu_context_destroy(lgpu_context_t ctx);
/* A context from the library's per-device free list (created when the list is
 * empty); release returns it with its scratch and pinned staging kept.  The
 * caller must have finished all work that uses the context before releasing
 * it (e.g. by synchronising the stream it used). */
lgpu_status_t lgpu_context_acquire(int device, lgpu_context_t *ctx);
lgpu_status_t lgpu_context_release(lgpu_context_t ctx);
/* Grow the context's scratch to at least `bytes` now (optional; reductions
 * grow it on first use). */
lgpu_status_t lgpu_context_reserve(lgpu_context_t ctx, size_t bytes);

/* ---- state preparation (initSV.cu:64-117; StateVectorCudaManaged.hpp:144-185;
 *      StateVectorCudaBase.hpp:234-240) */
/* sv = 0 everywhere except sv[index] = (re, im). */
lgpu_status_t lgpu_set_basis(void *sv, uint32_t n, lgpu_dtype_t dt, uint64_t index, double re,
                             double im, lgpu_stream_t stream);
/* Optionally zero sv, then sv[indices[i]] = values[i] (device arrays;
 * values of the state's dtype). */
lgpu_status_t lgpu_scatter(void *sv, uint32_t n, lgpu_dtype_t dt, const void *values,
                           const int64_t *indices, uint64_t count, int zero_first,
                           lgpu_stream_t stream);

/* ---- gates -------------------------------------------------------------- */
/* Dense controlled 2^t x 2^t matrix from HOST memory, t <= 12
 * (custatevecApplyMatrix at StateVectorCudaManaged.hpp:1433-1471, 1517-1555).
 * 1-target matrices are classified on the host (phase-only, diagonal,
 * permutation, real, RX-like, dense) and run the cheapest kernel body. */
lgpu_status_t lgpu_apply_matrix(void *sv, uint32_t n, lgpu_dtype_t dt, const double *matrix,
                                uint32_t t, const int32_t *tgts, uint32_t c, const int32_t *ctrls,
                                const int32_t *ctrl_vals, int adjoint, lgpu_stream_t stream);

/* The same gate applied to `nstates` states of equal size in one launch
 * (the adjoint sweep's bra updates, AdjointDiffGPU.hpp:279-319). */
lgpu_status_t lgpu_apply_matrix_multi(void *const *svs, uint32_t nstates, uint32_t n,
                                      lgpu_dtype_t dt, const double *matrix, uint32_t t,
                                      const int32_t *tgts, uint32_t c, const int32_t *ctrls,
                                      const int32_t *ctrl_vals, int adjoint,
                                      lgpu_stream_t stream);

/* exp(i * angle * P) for the Pauli word `paulis` (chars I,X,Y,Z) on tgts,
 * under controls (custatevecApplyPauliRotation at
 * StateVectorCudaManaged.hpp:1374-1385; the reference passes angle = -param/2,
 * or +param/2 for the adjoint). */
lgpu_status_t lgpu_apply_pauli_rotation(void *sv, uint32_t n, lgpu_dtype_t dt, double angle,
                                        uint32_t t, const int32_t *tgts, const char *paulis,
                                        uint32_t c, const int32_t *ctrls,
                                        const int32_t *ctrl_vals, lgpu_stream_t stream);

lgpu_status_t lgpu_apply_pauli_rotation_multi(void *const *svs, uint32_t nstates, uint32_t n,
                                              lgpu_dtype_t dt, double angle, uint32_t t,
                                              const int32_t *tgts, const char *paulis, uint32_t c,
                                              const int32_t *ctrls, const int32_t *ctrl_vals,
                                              lgpu_stream_t stream);

/* ---- fused gate blocks (shared-memory tiles) -------------------------------
 * Replaces the per-gate loop of the batched applyOperation overloads
 * (StateVectorCudaManaged.hpp:270-315), which issue one custatevecApplyMatrix
 * or custatevecApplyPauliRotation per operation; the C++ layer plans the
 * blocks (GateLowering.hpp).  No single reference call corresponds.
 * A block is a list of 1- and 2-target gates (controls allowed) whose target
 * bits all lie in the tile bit set.  One launch streams the state once:
 * each CTA loads a tile of 2^k amplitudes (the tile bits vary, every other bit
 * is fixed), applies all gates in order in shared memory and stores the tile.
 * Gate record layout (lgpu_fused_gate_t): see below. */
typedef struct {
    int32_t ntgt;      /* 1 or 2 */
    int32_t tgt[2];    /* state bits; tgt[0] = most significant matrix bit */
    int32_t nctrl;     /* 0..4 */
    int32_t ctrl[4];   /* state bits */
    int32_t ctrl_val[4];
    double m[32];      /* row-major 2^ntgt x 2^ntgt complex (interleaved) */
} lgpu_fused_gate_t;

/* tile_bits: k distinct state bits (k <= 13 for C64, <= 12 for C128); with
 * 0..m-1 the longest run of lowest state bits among them, at most 8 others.
 * Gates must target only tile bits (controls may be anywhere). */
lgpu_status_t lgpu_apply_fused_block(void *sv, uint32_t n, lgpu_dtype_t dt, uint32_t k,
                                     const int32_t *tile_bits, uint32_t ngates,
                                     const lgpu_fused_gate_t *gates, lgpu_stream_t stream);

/* ---- measurements ----------------------------------------------------------- */
/* <sv|M|sv> for a dense 2^t x 2^t host matrix on tgts,
 * t <= LGPU_MAX_EXPVAL_TARGETS (13: the reference's device sends Hamiltonians
 * on fewer than 14 wires as one dense matrix, lightning_gpu.py:856-861);
 * out = (re, im) (custatevecComputeExpectation at
 * StateVectorCudaManaged.hpp:1602-1639, 1674-1712).  The matrix is copied
 * into the context's scratch (up to 1 GiB for 13 targets). */
lgpu_status_t lgpu_expval_matrix(lgpu_context_t ctx, const void *sv, uint32_t n, lgpu_dtype_t dt,
                                 const double *matrix, uint32_t t, const int32_t *tgts,
                                 double *out, int out_on_device, lgpu_stream_t stream);

/* <P_j> for nwords Pauli words given as bit masks: flip = X|Y bits,
 * sign = Y|Z bits, ny = number of Y letters (custatevecComputeExpectationsOnPauliBasis
 * at StateVectorCudaManaged.hpp:1117-1128).  Words with equal flip masks are
 * evaluated in one pass.  out[j] = Re <P_j> (the imaginary part vanishes for a
 * normalised state); FP64 accumulation for both dtypes. */
lgpu_status_t lgpu_expval_pauli_words(lgpu_context_t ctx, const void *sv, uint32_t n,
                                      lgpu_dtype_t dt, uint32_t nwords, const uint64_t *flip,
                                      const uint64_t *sign, const uint8_t *ny, double *out,
                                      int out_on_device, lgpu_stream_t stream);

/* Marginal probabilities: out[idx] sums |sv_i|^2 over i whose bit bits[q]
 * equals bit q of idx (custatevecAbs2SumArray at StateVectorCudaManaged.hpp:957-967).
 * k <= 24. */
lgpu_status_t lgpu_probs(lgpu_context_t ctx, const void *sv, uint32_t n, lgpu_dtype_t dt,
                         uint32_t k, const int32_t *bits, double *out, int out_on_device,
                         lgpu_stream_t stream);

/* Inverse-CDF sampling (custatevecSampler* at StateVectorCudaManaged.hpp:1015-1035):
 * for each draw r in [0,1) return the smallest index i with
 * cdf_i > r * sum|sv|^2 (FP64 prefix sums); a draw past the end selects the last
 * index of non-zero probability.  draws and out_idx are HOST arrays; out_idx
 * is in draw order (the caller sorts for the reference's ascending order). */
lgpu_status_t lgpu_sample(lgpu_context_t ctx, const void *sv, uint32_t n, lgpu_dtype_t dt,
                          const double *draws, uint64_t shots, uint64_t *out_idx,
                          lgpu_stream_t stream);

/* <a|b> = sum conj(a_i) b_i, FP64 accumulation (cublasZdotc/Cdotc at
 * cuda_helpers.hpp:456-497); out = (re, im). */
lgpu_status_t lgpu_dot(lgpu_context_t ctx, const void *a, const void *b, uint32_t n,
                       lgpu_dtype_t dt, double *out, int out_on_device, lgpu_stream_t stream);

/* Allocation-free <a|b>: no counterpart in the reference.  Same result bits
 * as lgpu_dot, but the reduction scratch is a static device array of
 * lgpu_dot_static_scratch_bytes() (32 KiB) per device and a host `out` is
 * written by a direct copy, so the call allocates no device or host memory.
 * For callers that must not allocate: a state that fills the device leaves no
 * room for a context's scratch, and a context's first use or growth allocates
 * and synchronises the whole device.  The first call on a device looks up the
 * array's address (with that device current) and belongs before any stream
 * capture; lgpu_device_reset forgets the address, so the first call after a
 * reset looks it up again.  `stream` must belong to the current device
 * (LGPU_ERR_INVALID_ARG otherwise).  With a host `out` the call synchronises
 * `stream`.  Calls that can overlap on one device share the array and race:
 * order them.  A reduction whose grid needs more scratch than the array
 * holds is rejected with LGPU_ERR_INVALID_ARG. */
lgpu_status_t lgpu_dot_static(const void *a, const void *b, uint32_t n, lgpu_dtype_t dt,
                              double *out, int out_on_device, lgpu_stream_t stream);
size_t lgpu_dot_static_scratch_bytes(void);

/* y += alpha * x (cublasZaxpy/Caxpy at cuda_helpers.hpp:512-528). */
lgpu_status_t lgpu_axpy(double alpha_re, double alpha_im, const void *x, void *y, uint32_t n,
                        lgpu_dtype_t dt, lgpu_stream_t stream);
/* x *= alpha (cublasScalEx at cuda_helpers.hpp:544-560). */
lgpu_status_t lgpu_scale(double alpha_re, double alpha_im, void *x, uint32_t n, lgpu_dtype_t dt,
                         lgpu_stream_t stream);
/* dst = src over 2^n amplitudes (StateVectorCudaBase.hpp:104-219 D2D copies). */
lgpu_status_t lgpu_copy(void *dst, const void *src, uint32_t n, lgpu_dtype_t dt,
                        lgpu_stream_t stream);

/* out = sum_t coeff_t * P_t |in> for Pauli words (flip/sign/ny masks as in
 * lgpu_expval_pauli_words), one pass per distinct flip mask
 * (HamiltonianGPU::applyInPlace at ObservablesGPU.hpp:346-362). `in` and `out`
 * must not alias. */
lgpu_status_t lgpu_apply_pauli_sum(const void *in, void *out, uint32_t n, lgpu_dtype_t dt,
                                   uint32_t nterms, const double *coeffs /* complex, interleaved */,
                                   const uint64_t *flip, const uint64_t *sign, const uint8_t *ny,
                                   lgpu_stream_t stream);

/* CSR sparse matrix (2^n rows; int64 offsets/columns; values of the state
 * dtype; all device arrays).  y = H x (cusparseSpMV at ObservablesGPU.hpp:516-586)
 * and <x|H|x> (StateVectorCudaManaged.hpp:795-922). */
lgpu_status_t lgpu_spmv_csr(const int64_t *offsets, const int64_t *cols, const void *vals,
                            const void *x, void *y, uint32_t n, lgpu_dtype_t dt,
                            lgpu_stream_t stream);
lgpu_status_t lgpu_expval_csr(lgpu_context_t ctx, const int64_t *offsets, const int64_t *cols,
                              const void *vals, const void *x, uint32_t n, lgpu_dtype_t dt,
                              double *out, int out_on_device, lgpu_stream_t stream);

/* ---- adjoint sweep (AdjointDiffGPU.hpp:499-596) --------------------------------
 * One fused pass of the reverse sweep for one operation:
 *   out[k] = Im <bras[k]| G |ket>        (k < nbras; before the update)
 * then, if apply_udag != 0,  ket <- U^dag ket  and  bras[k] <- U^dag bras[k].
 * G and U are dense host matrices on the same bit set `bits` (w <= 4 bits,
 * bits[0] = most significant matrix bit); G may be NULL (no expectation).
 * `out` is a device array of nbras doubles (accumulated with '=' semantics). */
lgpu_status_t lgpu_adjoint_step(lgpu_context_t ctx, void *ket, void *const *bras, uint32_t nbras,
                                uint32_t n, lgpu_dtype_t dt, uint32_t w, const int32_t *bits,
                                const double *gen, const double *udag, int apply_udag,
                                double *out_dev, lgpu_stream_t stream);

/* The whole reverse sweep in one launch for states that fit in shared memory
 * (n <= lgpu_adjoint_sweep_max_qubits(dt): 12 for C128, 13 for C64): one CTA
 * per bra keeps lambda (from `ket`) and its bra in shared memory and runs
 * ops[0..nops) in the given order (the reverse of the circuit), each as
 *   jac[col * nbras + k] = Im <bra_k| G |lambda>   (when ng > 0)
 *   lambda <- U^dag lambda ;  bra_k <- U^dag bra_k
 * `ket` and `bras` are only read.  jac is a device array of at least
 * (max col + 1) * nbras doubles.  Same results as a sequence of
 * lgpu_adjoint_step calls; no counterpart in the reference. */
typedef struct {
    int32_t nu;       /* bits of U^dag: 1 or 2 (controls folded into the matrix) */
    int32_t ubits[2]; /* ubits[0] = most significant matrix bit */
    int32_t ng;       /* bits of the generator: 0 (no gradient), 1 or 2 */
    int32_t gbits[2];
    int32_t col;      /* Jacobian column of this operation (ng > 0) */
    double u[32];     /* U^dag, 2^nu x 2^nu row-major (re, im) */
    double g[32];     /* generator, 2^ng x 2^ng row-major (re, im) */
} lgpu_adj_op_t;

uint32_t lgpu_adjoint_sweep_max_qubits(lgpu_dtype_t dt);
lgpu_status_t lgpu_adjoint_sweep_small(lgpu_context_t ctx, const void *ket, void *const *bras,
                                       uint32_t nbras, uint32_t n, lgpu_dtype_t dt,
                                       const lgpu_adj_op_t *ops, uint32_t nops, double *jac_dev,
                                       lgpu_stream_t stream);

/* Several consecutive operations of the reverse sweep in one pass over the
 * states (states too large for lgpu_adjoint_sweep_small).  Each
 * step is a 1-target U^dag with controls and, when `gen_kind` >= 0, the
 * generator P1(controls) (x) g on the target:
 *   jac[col * jac_stride + k] = Im <bra_k| G |lambda>   (G on the pairs the
 *                                                        controls select)
 *   lambda <- U^dag lambda ;  bra_k <- U^dag bra_k
 * in step order.  Every target must be one of the k tile bits: the bits
 * 0..m-1 plus at most 6 others, k <= 11 (complex64: m >= 1).  nbras <= 2.
 * complex128 states are carried in float-float arithmetic inside the pass
 * (no FP64 instruction per pair), complex64 in FP32; the sums are
 * deterministic.  Replaces the per-operation
 * updateJacobian / applyOperationsAdj sequence of AdjointDiffGPU.hpp:560-595
 * for runs of such operations; no counterpart in the reference. */
typedef struct {
    int32_t tgt;         /* state bit */
    int32_t nctrl;       /* 0..2 */
    int32_t ctrl[2];     /* state bits */
    int32_t ctrl_val[2];
    int32_t gen_kind;    /* -1: no gradient; 0: dense g */
    int32_t col;         /* Jacobian column (gen_kind >= 0) */
    double u[8];         /* U^dag, 2x2 row-major (re, im) */
    double g[8];         /* generator on the target, 2x2 row-major (re, im) */
} lgpu_adj_block_step_t;

lgpu_status_t lgpu_adjoint_block(lgpu_context_t ctx, void *ket, void *const *bras, uint32_t nbras, uint32_t n,
                                 lgpu_dtype_t dt, uint32_t k, const int32_t *tile_bits,
                                 const lgpu_adj_block_step_t *steps, uint32_t nsteps, double *jac_dev,
                                 uint32_t jac_stride, lgpu_stream_t stream);

/* Float-float form of a complex128 state: each amplitude's 16 bytes hold the
 * floats (re.hi, im.hi, re.lo, im.lo), re = re.hi + re.lo to about 2^-47
 * relative.  A reverse sweep made of consecutive blocks keeps lambda and the
 * bras in this form between blocks, so each block skips the conversion of
 * its tiles: LGPU_FF_IN = the states arrive in float-float form, LGPU_FF_OUT
 * = leave them in it (complex128 only; 0 = lgpu_adjoint_block).  No other
 * call accepts a state in this form: lgpu_state_ff(sv, n, 0, stream) turns it
 * back into complex128, lgpu_state_ff(sv, n, 1, stream) converts the other
 * way; both in place, stream-ordered. */
#define LGPU_FF_IN 1u
#define LGPU_FF_OUT 2u
lgpu_status_t lgpu_adjoint_block_ff(lgpu_context_t ctx, void *ket, void *const *bras, uint32_t nbras, uint32_t n,
                                    lgpu_dtype_t dt, uint32_t k, const int32_t *tile_bits,
                                    const lgpu_adj_block_step_t *steps, uint32_t nsteps, double *jac_dev,
                                    uint32_t jac_stride, uint32_t ff_flags, lgpu_stream_t stream);
lgpu_status_t lgpu_state_ff(void *sv, uint32_t n, int to_ff, lgpu_stream_t stream);
/* lgpu_apply_fused_block with the same float-float flags (complex128 only): a
 * run of consecutive blocks keeps the state in float-float form from one
 * block to the next, so only the first block converts its tiles on load and
 * only the last converts them back on store. */
lgpu_status_t lgpu_apply_fused_block_ff(void *sv, uint32_t n, lgpu_dtype_t dt, uint32_t k,
                                        const int32_t *tile_bits, uint32_t ngates,
                                        const lgpu_fused_gate_t *gates, uint32_t ff_flags, lgpu_stream_t stream);

/* ---- CUDA graphs (stream capture) ------------------------------------------
 * Capture everything issued on `stream` between begin and end into an
 * executable graph; launch replays it on any stream.  No counterpart in the
 * reference (used by the batched-circuit executor and the serving loop). */
typedef struct lgpu_graph_s *lgpu_graph_t;
lgpu_status_t lgpu_graph_begin(lgpu_stream_t stream);
lgpu_status_t lgpu_graph_end(lgpu_stream_t stream, lgpu_graph_t *graph);
lgpu_status_t lgpu_graph_launch(lgpu_graph_t graph, lgpu_stream_t stream);
lgpu_status_t lgpu_graph_destroy(lgpu_graph_t graph);

/* ---- batched circuits (one persistent launch) --------------------------------
 * Many independent circuits run in one launch of a persistent kernel.  The
 * host lowers and fuses each circuit into blocks of gates whose targets fit a
 * shared-memory tile of 2^k amplitudes (k <= kmax; a circuit with n <= kmax
 * qubits is a single block holding the whole state) and uploads the records
 * below.  Gate matrices live in a device pool; parametric ones are rebuilt
 * from a device parameter array by lgpu_batch_prepare, so a captured graph
 * [params H2D, prepare, counter reset, run, results D2H] can be replayed with
 * new parameters.  No counterpart in the reference (it runs one circuit per
 * device call). */
typedef struct {
    uint8_t kind;      /* 0 dense 1q, 1 diagonal 1q, 2 X, 3 real 1q, 4 RX-like 1q, 5 dense 2q, 6 SWAP,
                          7 folded into the preceding chain head (skipped by the kernel) */
    uint8_t pkind;     /* 0 fixed matrix, 1 RX, 2 RY, 3 RZ, 4 PhaseShift, 5 Rot, 6 IsingXX, 7 IsingYY, 8 IsingZZ */
    uint8_t q0, q1;    /* tile positions of the targets, q0 = most significant matrix bit */
    uint32_t cmask;    /* controls inside the tile (tile positions) and their values */
    uint32_t cval;
    int32_t param;     /* index of the first parameter (-1: none) */
    uint32_t flags;    /* bit 0: adjoint (parametric gates); bit 1: chain head, whose matrix is the
                          product of the q1 gates recorded right after it */
    uint32_t mat;      /* offset of the gate's slot in the pool, in doubles (16 for 1q, 48 for 2q; the
                          C64 float copy of the matrix is written into the slot by lgpu_batch_prepare) */
    uint64_t omask;    /* controls outside the tile (state bits) and their values */
    uint64_t oval;
} lgpu_bgate_t;

typedef struct {
    uint32_t n, block_off, block_cnt, obs_off, obs_cnt, out;
} lgpu_bcircuit_t;

typedef struct {
    uint8_t k, m, pad0, pad1; /* tile bits, length of the low run 0..m-1 (k - m <= 6) */
    uint8_t bits[16];         /* sorted tile bits */
    uint32_t gate_off, gate_cnt;
} lgpu_bblock_t;

typedef struct {
    uint64_t tflip;  /* X|Y bits of the Pauli word in tile positions of the circuit's last block */
    uint64_t sign;   /* Y|Z bits (state bits) */
    double cr, ci;   /* coefficient * i^(number of Y) */
} lgpu_bterm_t;

typedef struct {
    const lgpu_bcircuit_t *circuits;
    const uint32_t *order;   /* processing order (NULL: identity) */
    uint32_t ncircuits;
    uint32_t kmax;           /* circuits of n <= kmax qubits run entirely in shared memory,
                                kmax <= 13 (C128) / 14 (C64) */
    const lgpu_bblock_t *blocks;
    const lgpu_bgate_t *gates;
    const double *pool;
    const lgpu_bterm_t *terms;
    void *scratch;           /* grid * scratch_amps amplitudes (states above kmax qubits) */
    uint64_t scratch_amps;
    unsigned *counter;       /* work-queue counter, zero before each launch */
    double *out;             /* one result per circuit */
    uint32_t threads;        /* 128, 256 or 512 */
    uint32_t klarge;         /* tile bits of circuits above kmax qubits, <= 12 (C128) / 13 (C64);
                                their tiles stream through a 3-stage shared-memory ring */
} lgpu_batch_args_t;

lgpu_status_t lgpu_batch_prepare(const lgpu_bgate_t *gates, uint64_t ngates, const double *params, double *pool,
                                 lgpu_dtype_t dt, lgpu_stream_t stream);
lgpu_status_t lgpu_batch_run(const lgpu_batch_args_t *args, lgpu_dtype_t dt, unsigned grid, lgpu_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* LGPU_H */
