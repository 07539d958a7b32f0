/*
 * qsgb.h -- C ABI of the GB300 density-matrix (Pauli vector) kernels.
 *
 * Every entry point takes plain device pointers, 64-bit sizes and a CUDA
 * stream (as `void*`, NULL = legacy default stream), launches asynchronously
 * on that stream and returns an int status (QSGB_OK == 0).  Argument errors
 * are detected on the host before any launch.  No entry point allocates
 * device memory; the ones that need scratch space take it from the caller
 * and report the size they need through a *_scratch_bytes() query.
 *
 * Data model (quantumsim/pauli_vectors/pauli_vector.py:6-72): a Pauli vector
 * over n qudits is a dense C-order tensor of shape (d_0, ..., d_{n-1}),
 * qudit 0 most significant, d_i = dim_pauli of qudit i (1..d_hilbert^2).
 * Element types: QSGB_F64 (IEEE double) or QSGB_F32 (IEEE float).
 *
 * Kernels that take an `unsigned* dev_status` (may be NULL) OR device-side
 * status bits (QSGB_DEV_*) into it; the host reads it at its next sync.
 */
#ifndef QSGB_H_
#define QSGB_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (host return values) ---- */
#define QSGB_OK 0
#define QSGB_ERR_INVALID 1     /* bad argument (shape, pointer, flag) */
#define QSGB_ERR_CUDA 2        /* a CUDA runtime call failed */
#define QSGB_ERR_UNSUPPORTED 3 /* valid request the library does not serve */
#define QSGB_ERR_SCRATCH 4     /* caller scratch buffer too small */

/* ---- device status bits (written into *dev_status) ---- */
#define QSGB_DEV_RANGE 1u      /* reserved: apply kernels no longer raise it --
                                  float-float rows whose inputs or results
                                  leave the float pair's range are computed
                                  again in native FP64 by the kernel */
#define QSGB_DEV_TIMEOUT 2u    /* a bounded device-side wait gave up */
#define QSGB_DEV_BADITEM 4u    /* batched work queue met a malformed item
                                  (unknown op, targets outside its instance,
                                  range past its vector); it was skipped */

/* ---- storage element types ---- */
#define QSGB_F64 0
#define QSGB_F32 1

/* ---- arithmetic of apply_ptm ---- */
#define QSGB_ARITH_AUTO 0  /* F64 storage -> DF64; F32 storage -> F32 */
#define QSGB_ARITH_DF64 1  /* float-float (48-bit significand) on the FP32
                              pipes; single-term rows use one FP64 multiply */
#define QSGB_ARITH_F64 2   /* native FP64 FMA (exact IEEE, slow on GB300) */
#define QSGB_ARITH_F32 3   /* FP32 FMA (F32 storage only) */
#define QSGB_ARITH_TC 4    /* F64 storage: every dense-shaped 16 x 16 host
                              PTM (two full-basis qubits) on the tensor
                              cores (FP64 values split into FP16 digit
                              planes, exact FP32 sums); other PTMs as AUTO.
                              AUTO itself sends 16 x 16 host PTMs with more
                              than 8 non-zero terms per row there */

/* ---- PTM layout flags ---- */
#define QSGB_PTM_SWAPPED 1    /* 2-qudit PTM given in order (less significant,
                                 more significant) qudit: the reference's
                                 `qubit0 > qubit1` case, cuda.py:171-173 */
#define QSGB_PTM_TRANSPOSED 2 /* apply the transpose of the stored PTM
                                 (adjoint / gradient w.r.t. the state) */
#define QSGB_PTM_HOST 4       /* `ptm` is a HOST pointer, read during the
                                 call (no device copy, no allocation).  Its
                                 sparsity pattern selects a kernel compiled
                                 for that pattern at run time (NVRTC, cached);
                                 without NVRTC, PTMs of <= 256 entries run in
                                 the generic kernel, larger ones return
                                 QSGB_ERR_UNSUPPORTED */
#define QSGB_PTM_NOJIT 8      /* never use the run-time specialised kernel */

/* Version of this ABI (bumped on any signature change). */
int qsgb_abi_version(void);

/* Human-readable text for a status code (static storage). */
const char* qsgb_status_string(int status);

/* 1 if run-time specialisation of apply kernels (NVRTC) is available (and
 * not disabled by the environment variable QSGB_NO_JIT), else 0. */
int qsgb_jit_available(void);

/*
 * One-qudit PTM application.
 * Replaces: quantumsim/pauli_vectors/cuda.py:223-277 (_apply_single_qubit_ptm
 * launching primitives.cu:15-89 with dim_a_in = 1) and
 * quantumsim/pauli_vectors/numpy.py:50-64 (np.einsum).
 *
 *   out[y, r, z] = sum_k P[r, k] * in[y, k, z]
 *
 * in  : tensor viewed as (dim_y, d_in, dim_z), `dtype` elements
 * out : tensor viewed as (dim_y, d_out, dim_z); must not alias `in`
 * ptm : FP64 matrix, row-major (d_out, d_in), on the device (or on the host
 *       with QSGB_PTM_HOST); with QSGB_PTM_TRANSPOSED it is stored as
 *       (d_in, d_out) and its transpose is applied
 * max_terms : upper bound on the number of non-zero entries of a device
 *       PTM (d_out*d_in or 0 is always safe; smaller values shrink shared
 *       memory); ignored for a host PTM, whose entries the call counts
 */
int qsgb_apply_ptm1(const void* in, void* out, const double* ptm,
                    int64_t d_out, int64_t d_in, int64_t dim_y, int64_t dim_z,
                    int ptm_flags, int dtype, int arith, int64_t max_terms,
                    unsigned* dev_status, void* stream);

/*
 * Two-qudit PTM application on qudits a < b (a more significant).
 * Replaces: quantumsim/pauli_vectors/cuda.py:151-221 (_apply_two_qubit_ptm,
 * primitives.cu:15-89 two_qubit_general_ptm) and numpy.py:50-64.
 *
 *   out[x, ra, y, rb, z] = sum_{ka,kb} P[ra, rb, ka, kb] * in[x, ka, y, kb, z]
 *
 * in  : viewed as (dim_x, d0_in, dim_y, d1_in, dim_z)
 * out : viewed as (dim_x, d0_out, dim_y, d1_out, dim_z); must not alias `in`
 * ptm : FP64 (device, or host with QSGB_PTM_HOST), row-major
 *       (d0_out, d1_out, d0_in, d1_in), index 0 =
 *       qudit a.  QSGB_PTM_SWAPPED: stored as (d1_out, d0_out, d1_in, d0_in).
 *       QSGB_PTM_TRANSPOSED: stored as the forward PTM (in/out exchanged).
 */
int qsgb_apply_ptm2(const void* in, void* out, const double* ptm,
                    int64_t d0_out, int64_t d1_out, int64_t d0_in,
                    int64_t d1_in, int64_t dim_x, int64_t dim_y, int64_t dim_z,
                    int ptm_flags, int dtype, int arith, int64_t max_terms,
                    unsigned* dev_status, void* stream);

/*
 * Compile ahead of time the kernel that qsgb_apply_ptm2 (or, with d0_out =
 * d0_in = dim_x = 1, qsgb_apply_ptm1) would specialise at run time to this
 * host PTM (QSGB_PTM_HOST required) and geometry, for tensors aligned as
 * device allocators return them; nothing is launched and no tensor is
 * touched.  Safe to call from several host threads at once, which compile
 * in parallel: a circuit's distinct sparsity patterns can be prepared
 * together instead of one by one at first use.  QSGB_OK when the kernel is
 * ready, QSGB_ERR_UNSUPPORTED when the call would not use a specialised
 * kernel (nothing to prepare).
 * No counterpart in the reference (PyCUDA compiles its one kernel once).
 */
int qsgb_prepare_ptm2(const double* ptm, int64_t d0_out, int64_t d1_out,
                      int64_t d0_in, int64_t d1_in, int64_t dim_x,
                      int64_t dim_y, int64_t dim_z, int ptm_flags, int dtype,
                      int arith);

/*
 * Diagnostic: generate the CUDA source of the kernel that qsgb_prepare_ptm2
 * would compile for this host PTM and geometry, and compile it with NVRTC
 * for sm_103a without loading it -- no device is needed, so a build host can
 * check the code generator.  The source text (NUL-terminated, truncated to
 * src_bytes - 1 characters) is written to `src` when it is not NULL.
 * QSGB_OK when it compiles, QSGB_ERR_CUDA on a compile error (the NVRTC log
 * goes to stderr when the environment sets QSGB_JIT_VERBOSE),
 * QSGB_ERR_UNSUPPORTED when no specialised kernel applies or NVRTC is
 * missing.  No counterpart in the reference.
 */
int qsgb_jit_check_ptm2(const double* ptm, int64_t d0_out, int64_t d1_out,
                        int64_t d0_in, int64_t d1_in, int64_t dim_x,
                        int64_t dim_y, int64_t dim_z, int ptm_flags,
                        int dtype, int arith, char* src, int64_t src_bytes);

/*
 * Multi-axis take ("multitake"): out = in[np.ix_(idx_0, ..., idx_{n-1})].
 * Replaces: quantumsim/pauli_vectors/primitives.cu:100-130 (multitake, used by
 * cuda.py:279-345 diagonal()).  Index lists are CSR-like as in cuda.py:307-313
 * but HOST arrays (copied into the launch): idx_off[ndim+1] offsets into
 * idx[].  An index of -1 writes 0 (a basis element absent from a subbasis).
 * in_dtype / out_dtype may differ (F32 -> F64 widening for diagonals).
 * ndim <= 32, idx_off[ndim] <= 2048.
 */
int qsgb_gather(const void* in, void* out, int in_dtype, int out_dtype,
                int ndim, const int64_t* in_shape, const int32_t* idx_off,
                const int32_t* idx, void* stream);

/*
 * Take along one axis: out[o, j, i] = in[o, idx[j], i] for a tensor viewed as
 * (outer, d_in, inner).  The per-qudit basis reduction (`reduce_basis`, e.g.
 * 9 -> 3 with the computational subbasis) and `project` (-> 1 element).
 * Reference semantics: apply_ptm of the selection PTM eye(d_in)[idx]
 * (quantumsim/operations/operation.py:549-551, bases/pauli_basis.py:70-89).
 * idx: HOST array of d_out entries (copied into the launch), -1 writes 0.
 * Bit-exact copy.  d_out <= 2048.
 */
int qsgb_take_axis(const void* in, void* out, int dtype, int64_t outer,
                   int64_t d_in, int64_t inner, const int32_t* idx,
                   int64_t d_out, void* stream);

/*
 * Marginal probabilities from an FP64 diagonal (the DM diagonal, shape
 * `shape[0..ndim)` C order): out[j] = sum of diag entries whose index along
 * axis `axis` equals j, j < shape[axis]; axis == -1 gives the trace in
 * out[0].  Deterministic two-stage reduction with FP64 accumulation.
 * Replaces: cuda.py:355-384 (meas_prob: one ReductionKernel launch per
 * outcome) and cuda.py:347-349 (trace: D2H + np.sum); numpy.py:82-84,97-107.
 * scratch: device buffer of qsgb_marginals_scratch_bytes(...) bytes.
 */
int64_t qsgb_marginals_scratch_bytes(int64_t n, int64_t n_out);
int qsgb_marginals(const double* diag, int ndim, const int64_t* shape,
                   int axis, double* out, void* scratch, int64_t scratch_bytes,
                   void* stream);

/*
 * qsgb_marginals without caller scratch and without any allocation.
 *
 * No counterpart in the reference.  Some programs that embed this library
 * cannot allocate device memory when they need probabilities: an
 * application whose device memory is wholly owned by its own pool allocator
 * (and which forbids outside cudaMalloc calls), or a latency-critical
 * measurement loop in which the implicit device synchronisation of
 * cudaMalloc / cudaFree would stall the pipeline.  This entry point computes
 * exactly what qsgb_marginals computes, but keeps its partial sums in a
 * fixed 128 KiB array inside the library (a file-scope __device__ array that
 * every GPU loading the library holds until the process exits).  It calls
 * no cudaMalloc, cudaFree or allocating library routine.
 *
 * - The first call on each device looks up the array's device address
 *   (cudaGetSymbolAddress) with that device current.  Under CUDA's default
 *   lazy module loading that lookup also loads the library's device code
 *   on the device, which is when the 128 KiB array is reserved: a program
 *   whose pool has already taken every byte of device memory can see that
 *   first call fail with QSGB_ERR_CUDA.  Make one warm-up call per device
 *   at initialisation, before the pool takes its memory and before any
 *   stream capture on the device.
 * - The address is cached per device and CUDA context.  After
 *   cudaDeviceReset, or in another context made current through the driver
 *   API, the next call looks it up again (the same first-call rules apply).
 * - Requests needing more than qsgb_marginals_noalloc_max_scratch_bytes()
 *   of partial sums (chunks x outcomes > 16384 doubles) return
 *   QSGB_ERR_SCRATCH; up to 32 outcomes per axis always fit.
 * - All calls share the one array and it keeps the last call's contents
 *   (every partial a call reads is written by that call first, so nothing
 *   needs clearing).  Calls that can overlap on the GPU -- on different
 *   streams, or from different host threads -- race on the array; serialise
 *   them (one stream, or events).
 */
int64_t qsgb_marginals_noalloc_max_scratch_bytes(void);
int qsgb_marginals_noalloc(const double* diag, int ndim, const int64_t* shape,
                           int axis, double* out, void* stream);

/*
 * Marginals of the DM diagonal read straight from the Pauli vector: the
 * diagonal is the multitake of qsgb_gather (same host index lists; -1
 * selects a zero), and out[j] = sum of its entries whose index along `axis`
 * is j (j < number of indices of `axis`), or out[0] = the trace for
 * axis == -1.  One launch, deterministic, FP64 accumulation for FP64 and
 * FP32 vectors.  out[n_out] receives the value of the device status word
 * *dev_status (0 when dev_status is NULL) as it stands when the kernel runs,
 * so a single device-to-host copy of n_out + 1 doubles returns the result
 * and every earlier kernel's status bits.  With host_out != NULL the call
 * also makes that copy into host_out (pinned memory for an asynchronous
 * copy) and waits for it on the stream before returning; with NULL it
 * returns at once, the results on the device.  Diagonals of at most 2^22 entries
 * and axes of at most 64 indices; larger ones return QSGB_ERR_UNSUPPORTED
 * (use qsgb_gather and qsgb_marginals).  Without scratch (below) one block
 * does the whole reduction.
 * Replaces: cuda.py:347-384 (trace and meas_prob: multitake, then a host
 * sum or one ReductionKernel launch and device sync per outcome) and
 * numpy.py:82-84, 97-107.
 */
int qsgb_diag_marginals(const void* in, int in_dtype, int ndim,
                        const int64_t* in_shape, const int32_t* idx_off,
                        const int32_t* idx, int axis, double* out,
                        const unsigned* dev_status, double* host_out,
                        void* scratch, int64_t scratch_bytes, void* stream);
/* Scratch for qsgb_diag_marginals to spread a large diagonal over up to one
 * block per SM: a 16-byte-aligned device buffer whose first 16 bytes are
 * zero before its first use (each call leaves them zero again), of this many
 * bytes (fewer bytes, or scratch == NULL, use fewer blocks, down to one).
 * The last block to finish adds the per-block partials in block order, so
 * results stay deterministic for a given device.  Calls that share a
 * scratch buffer must not overlap on the GPU. */
int64_t qsgb_diag_marginals_scratch_bytes(void);

/*
 * Partial trace: out[kept...] = sum over traced qudits t of
 *   in[...] * prod_t w_t[k_t]
 * with w_t[k] = Re tr(P_k) of qudit t's basis (numpy.py:86-95).  Kept
 * qudits appear in ascending order in `out`.  keep[i] != 0 keeps qudit i.
 * weights: HOST array, the concatenation of w_t over traced qudits in
 * ascending order (copied into the launch; zero weights are skipped).
 * FP64 accumulation for both storage types; out has the `dtype` of in.
 */
int qsgb_partial_trace(const void* in, void* out, int dtype, int ndim,
                       const int64_t* shape, const int32_t* keep,
                       const double* weights, void* stream);

/* x[i] *= alpha for i < n (renormalize: numpy.py:109-117, cuda.py:386-395) */
int qsgb_scale(void* x, int dtype, int64_t n, double alpha, void* stream);

/*
 * x[i] *= 1 / *denom (device scalar) when *denom > threshold, else x is
 * left unchanged.  Renormalisation without a host round trip.
 */
int qsgb_scale_by_inverse(void* x, int dtype, int64_t n, const double* denom,
                          double threshold, void* stream);

/*
 * Gradient of apply_ptm with respect to the PTM (reverse mode):
 *   dP[r, k] = sum_{groups} g_out[..., r, ...] * x_in[..., k, ...]
 * a tall-skinny reduction over the bystander index, FP64 accumulation.
 * dptm: device FP64 (d_out, d_in) [1 qudit] or (d0o, d1o, d0i, d1i)
 * [2 qudits, qudit a first], overwritten.  The state gradient uses
 * qsgb_apply_ptm* with QSGB_PTM_TRANSPOSED.
 * scratch: qsgb_ptm_grad_scratch_bytes(n_groups, k_out, k_in) bytes.
 */
int64_t qsgb_ptm_grad_scratch_bytes(int64_t n_groups, int64_t k_out,
                                    int64_t k_in);
int qsgb_ptm_grad1(const void* x_in, const void* g_out, double* dptm,
                   int64_t d_out, int64_t d_in, int64_t dim_y, int64_t dim_z,
                   int dtype, void* scratch, int64_t scratch_bytes,
                   void* stream);
int qsgb_ptm_grad2(const void* x_in, const void* g_out, double* dptm,
                   int64_t d0_out, int64_t d1_out, int64_t d0_in,
                   int64_t d1_in, int64_t dim_x, int64_t dim_y, int64_t dim_z,
                   int dtype, void* scratch, int64_t scratch_bytes,
                   void* stream);

/* ===================================================================
 * Batched execution: many independent circuits (FP32 Pauli vectors of
 * qubits in the full 4-element basis) forward AND adjoint in ONE persistent
 * launch.  No counterpart in the reference (it runs one circuit at a time
 * through Python).  The program is a list of stages; a stage is a list of
 * work items whose instances are independent; persistent blocks take items
 * from a per-stage counter and meet at a grid barrier between stages.
 * =================================================================== */
#define QSGB_BOP_INIT 1     /* x[beg:end) = |0..0> (1 at element 0, else 0) */
#define QSGB_BOP_ZERO_G 2   /* g[beg:end) = 0 */
#define QSGB_BOP_APPLY 3    /* x = P x on groups [beg, end), in place */
#define QSGB_BOP_SAVE 4     /* ckpt[ptm][beg:end) = x[beg:end) */
#define QSGB_BOP_RESTORE 5  /* x[beg:end) = ckpt[ptm][beg:end) */
#define QSGB_BOP_LOSS 6     /* whole instance: prob = diag(x) (FP64),
                               loss = KL(target || prob), g[diag] = dloss/dprob */
#define QSGB_BOP_ADJOINT 7  /* groups [beg, end): x = P^-1 x, g = P^T g, and
                               grad_partial[slot] = sum g_out (x) x_in (FP64) */
#define QSGB_BOP_GRADSUM 8  /* grad[ptm] = sum of grad_partial[beg:end) */

typedef struct {
  float* x;           /* state, 4^n floats */
  float* g;           /* adjoint state, 4^n floats */
  float* ckpt;        /* checkpoint slots, 4^n floats each */
  int64_t size;       /* 4^n */
  int32_t n_qubits;   /* 1 <= n <= 16 */
  int32_t diag_offset;/* offset of this instance's 2^n entries in target/prob */
} qsgb_batch_instance;

typedef struct {
  int32_t op;         /* QSGB_BOP_* */
  int32_t inst;       /* instance index, below the program's n_instances */
  int32_t q0, q1;     /* target qubits, q0 < q1; q1 = -1 for one qubit */
  int32_t ptm;        /* PTM index (APPLY/ADJOINT/GRADSUM) or checkpoint slot */
  int32_t slot;       /* gradient partial slot (ADJOINT) */
  int64_t beg, end;   /* group, element or slot range */
} qsgb_batch_item;

typedef struct {
  const qsgb_batch_instance* instances; /* device */
  const qsgb_batch_item* items;         /* device */
  const int32_t* stage_begin;           /* device, n_stages + 1 item offsets */
  int32_t n_stages;
  int32_t n_instances;     /* entries of `instances`; items must index below it
                              (ABI version 2; fills what was padding) */
  uint32_t* work;          /* device, n_stages + 3 words, ZERO before each run */
  const float* ptm;        /* device, n_ptm x 256: P (sorted qubit order,
                              row-major out x in; 4x4 in the first 16) */
  const float* ptm_inv;    /* device, n_ptm x 256: P^-1 (ADJOINT) */
  double* grad_partial;    /* device, n_slots x 256 */
  double* grad;            /* device, n_ptm x 256 */
  const double* target;    /* device, sum of 2^n over instances */
  double* prob;            /* device, same layout as target */
  double* loss;            /* device, per instance */
} qsgb_batch_program;

/* Largest grid (blocks of `block` threads) whose blocks are all resident. */
int qsgb_batch_max_grid(int block);

/* Run a batch program.  grid <= qsgb_batch_max_grid(block); block = 256.
 * cooperative != 0 launches cooperatively (co-residency guaranteed).  Every
 * grid barrier spins at most `spin_limit` polls; on expiry the kernel sets
 * QSGB_DEV_TIMEOUT in *dev_status and all blocks return. */
int qsgb_batch_run(const qsgb_batch_program* prog, int grid, int block,
                   int cooperative, unsigned* dev_status, int64_t spin_limit,
                   void* stream);

#ifdef __cplusplus
}
#endif

#endif /* QSGB_H_ */
