/*
 * paraht.h -- C ABI of the GB300 (sm_103a) two-stage Hessenberg-triangular reduction.
 *
 * Reduces a real pencil (A, B), B upper triangular, to (H, T) = (Q^T A Z, Q^T B Z) with H upper
 * Hessenberg and T upper triangular, in two stages:
 *   stage 1  (A, B) -> (r-Hessenberg, triangular)    replaces ab2rht_simple, src/ab2rht.f90:8
 *   stage 2  r-Hessenberg -> Hessenberg              replaces rht2ht_householder, src/rht2ht.f90:1346
 * Q and Z are ACCUMULATED: both stages right-multiply the Q and Z they receive (pass identity
 * matrices for the plain transforms), exactly as the reference does.
 *
 * Layout: column-major FP64 with leading dimensions, like the reference's Fortran arrays
 * A(lda,*).  All integers are plain C ints passed by value (a Fortran caller uses bind(C) with
 * the VALUE attribute; see the Fortran module shipped with the library).
 *
 * Errors: every entry point returns an int status, 0 on success.  A negative value -i in
 * [-20,-1] names the invalid i-th argument, as LAPACK's INFO does; values <= -1000 are the
 * PARAHT_ERR_* codes below.  The reference has no error reporting (LAPACK INFO is ignored,
 * src/ab2rht.f90:105, :291); nothing here aborts the process.
 *
 * Valid parameters (checked): n >= 0 (0: nothing to do); 1 <= r <= 64; p >= 2; 1 <= nq <= r.  Stage 2 must be
 * given the same r that stage 1 used (src/profilereduction.f90:136, :144).  nq > r lies
 * outside the domain where the reference's staircase bookkeeping (src/rht2ht.f90:1649-1675,
 * :1823-1829) stays consistent: its results lose accuracy for some n, so it is rejected.
 *
 * Threading: entry points taking a paraht_ctx are thread-safe per context (one stream per
 * context, no global state).  The context-free host entry points use one lazily created
 * context per calling host thread on the current CUDA device.
 */
#ifndef PARAHT_H
#define PARAHT_H

#ifdef __cplusplus
extern "C" {
#endif

#define PARAHT_VERSION 100 /* 1.0.0 */

/* ---- status codes ---- */
#define PARAHT_OK 0
#define PARAHT_ERR_CUDA (-1001)          /* a CUDA runtime call failed */
#define PARAHT_ERR_ALLOC (-1002)         /* device or pinned-host allocation failed */
#define PARAHT_ERR_TIMEOUT (-1003)       /* a bounded device-side wait expired */
#define PARAHT_ERR_NONFINITE (-1004)     /* NaN/Inf found in the input (PARAHT_FLAG_CHECK_FINITE) */
#define PARAHT_ERR_NOT_SUPPORTED (-1005) /* parameter combination not supported on this device */
#define PARAHT_ERR_NO_DEVICE (-1006)     /* no usable CUDA device */
#define PARAHT_ERR_BAD_CTX (-1007)       /* null or destroyed context */
#define PARAHT_ERR_TOO_LARGE (-1008)     /* exceeds the fixed scratch of paraht_rht2ht_d_noalloc */

/* ---- flags (bit set) ---- */
#define PARAHT_FLAG_TIME_COMPONENTS 1 /* record per-phase times (time_components, src/ab2rht.f90:13) */
#define PARAHT_FLAG_CHECK_FINITE 2    /* reject non-finite inputs before reducing */
#define PARAHT_FLAG_SPLIT 4           /* split-precision (emulated FP64) bulk updates */
#define PARAHT_FLAG_NO_ZERO_FILL 8    /* keep roundoff below the structure instead of exact zeros */
#define PARAHT_FLAG_SEQUENTIAL 16     /* debug: run the stage-2 sweeps of a group one after the other in
                                         one CTA and all updates on one stream (the reference's order);
                                         results are bitwise identical to the default pipelined schedule */
#define PARAHT_FLAG_KERNEL_TIMES 32   /* time every bulk compact-WY op-list launch (split-precision or FP64)
                                         with CUDA events and count its algorithmic work
                                         (paraht_ctx_kernel_stats) */

#define PARAHT_FLAG_GIVENS 128     /* stage 2 by Givens rotations (rht2ht_givens, src/rht2ht.f90:696-1344)
                                         instead of small reflectors; needs r <= 32 and r + nq <= 64 */
#define PARAHT_FLAG_TIME_CHAIN 256 /* record the phase times on the critical-path stream of each stage
                                      without serialising the side streams: the phases then add up to the
                                      overlapped call's device time, each one holding the time the
                                      critical path spent in it, its waits for side streams included */

typedef struct paraht_ctx_s* paraht_ctx;

/* ---- context ---- */
int paraht_ctx_create(paraht_ctx* ctx, int device);
int paraht_ctx_destroy(paraht_ctx ctx);
/* Use an existing cudaStream_t (passed as void*); NULL selects the context's own stream. */
int paraht_ctx_set_stream(paraht_ctx ctx, void* stream);
/* Phase times of the last call, in seconds, when PARAHT_FLAG_TIME_COMPONENTS (phases run one after
 * the other) or PARAHT_FLAG_TIME_CHAIN (critical-path shares of the overlapped run) was set:
 *   [0] stage-1 left generation  [1] stage-1 right generation  [2] stage-1 multiplications
 *   [3] stage-2 generation       [4] stage-2 lookahead          [5] stage-2 application
 *   [6] host<->device copies (host entry points only)             [7] total device time
 * (the groups printed by src/ab2rht.f90:487-490 and src/rht2ht.f90:2044-2047). */
int paraht_ctx_phase_times(paraht_ctx ctx, double* times, int ntimes);
/* Number of GPU kernels the library launched during the last call on this context. */
int paraht_ctx_launch_count(paraht_ctx ctx, long long* count);
/* Largest absolute entry found below the structure (r-Hessenberg / Hessenberg for A,
 * triangular for B) before it was zeroed by the last call: [0] A, [1] B. */
int paraht_ctx_fill_residue(paraht_ctx ctx, double* residue, int nres);
/* With PARAHT_FLAG_KERNEL_TIMES, for the bulk compact-WY op-list kernels of the last call (the
 * split-precision kernel under PARAHT_FLAG_SPLIT, else the FP64 kernels; the FP64 path's 8-row
 * critical-path lists are not timed): [0] summed launch durations (s), [1] launches,
 * [2] algorithmic FP64-equivalent flops (4 len k per strip row per op, 2 len^2 for the Givens
 * stage's dense ops) of the stage-1 lists; [3..5] the same for the stage-2 lists; [6], [7] the
 * time during which at least one stage-1 / stage-2 list ran (the union of the launch intervals:
 * lists on different streams overlap, so their durations add up to more than the elapsed time).
 * No counterpart in the reference. */
int paraht_ctx_kernel_stats(paraht_ctx ctx, double* stats, int nstats);

/* ---- host-pointer drop-ins (copy in, reduce on the GPU, copy out) ----
 * paraht_ab2rht  <-> ab2rht_simple(n, A, lda, B, ldb, Q, ldq, Z, ldz, nb, p, time_components)
 *                    src/ab2rht.f90:8-13
 * paraht_rht2ht  <-> rht2ht_householder(n, A, lda, B, ldb, Q, ldq, Z, ldz, r, nq, time_components)
 *                    src/rht2ht.f90:1346-1351
 * paraht_reduce  <-> the two calls in sequence, src/profilereduction.f90:136 and :144
 * time_components is a C int (0/1) in place of the Fortran LOGICAL. */
int paraht_ab2rht(int n, double* A, int lda, double* B, int ldb, double* Q, int ldq, double* Z, int ldz, int nb,
                  int p, int time_components);
int paraht_rht2ht(int n, double* A, int lda, double* B, int ldb, double* Q, int ldq, double* Z, int ldz, int r,
                  int nq, int time_components);
int paraht_reduce(int n, double* A, int lda, double* B, int ldb, double* Q, int ldq, double* Z, int ldz, int r,
                  int p, int nq, int flags);

/* paraht_rht2ht_givens <-> rht2ht_givens(n, A, lda, B, ldb, Q, ldq, Z, ldz, r, nq)
 *                          src/rht2ht.f90:696-700 (the reference's stage-2 variant with Givens
 * rotations: the bulge chase needs no RQ, the rotations of a group are accumulated into
 * (r+nq) x (r+nq) orthogonal blocks and applied as dense products).  The same H, T as
 * paraht_rht2ht up to the signs of rows and columns.  r <= 32 and r + nq <= 64, else
 * PARAHT_ERR_NOT_SUPPORTED.  The device and combined entry points take PARAHT_FLAG_GIVENS. */
int paraht_rht2ht_givens(int n, double* A, int lda, double* B, int ldb, double* Q, int ldq, double* Z, int ldz, int r,
                         int nq);

/* Same, on an explicit context (host pointers). */
int paraht_reduce_host(paraht_ctx ctx, int n, double* A, int lda, double* B, int ldb, double* Q, int ldq, double* Z,
                       int ldz, int r, int p, int nq, int flags);

/* ---- device-pointer variants: arrays already resident in device memory, no copies;
 * work is enqueued on the context's stream and the call returns after it completes. ---- */
int paraht_ab2rht_d(paraht_ctx ctx, int n, double* A, int lda, double* B, int ldb, double* Q, int ldq, double* Z,
                    int ldz, int nb, int p, int flags);
int paraht_rht2ht_d(paraht_ctx ctx, int n, double* A, int lda, double* B, int ldb, double* Q, int ldq, double* Z,
                    int ldz, int r, int nq, int flags);
int paraht_reduce_d(paraht_ctx ctx, int n, double* A, int lda, double* B, int ldb, double* Q, int ldq, double* Z,
                    int ldz, int r, int p, int nq, int flags);

/* ---- stage 2 without any allocation.  No counterpart in the reference.
 * For callers that must not allocate device memory during the call (an application that owns
 * all device memory through its own pool, or code running where a cudaMalloc would synchronise
 * the device): same arithmetic and results as paraht_rht2ht_d (FP64 only), but the scratch
 * (reflector stores, progress words) lives in a fixed file-scope device array of
 * PARAHT_NOALLOC_SCRATCH_BYTES bytes instead of the context's workspace, so the call performs
 * no cudaMalloc/cudaFree and creates no events.
 * Size limit: the scratch needed is
 *     32 b nq (r + 2 nq + 1) + 4 (nq + 2) + 4096 bytes,  b = max(1, ceil((n-1)/r)) + 2,
 * which must not exceed PARAHT_NOALLOC_SCRATCH_BYTES (n <= 5313 for r = nq = 16, 15841 for
 * r = 16, nq = 8, 1217 for r = nq = 64); larger inputs return PARAHT_ERR_TOO_LARGE.
 * Flags: only PARAHT_FLAG_CHECK_FINITE, PARAHT_FLAG_NO_ZERO_FILL and PARAHT_FLAG_SEQUENTIAL are
 * accepted; any other bit returns PARAHT_ERR_NOT_SUPPORTED.  The scratch is shared by all
 * callers on a device and keeps the last call's contents; the library serialises the calls that
 * host threads of one process make, and work that overlaps a call on the GPU and uses the same
 * array (a graph or stream replaying such a call) races with it.  Every call looks up the
 * array's device address (cudaGetSymbolAddress) with its context's device current.  Everything
 * that must start at zero is cleared on the stream by the call itself. ---- */
#define PARAHT_NOALLOC_SCRATCH_BYTES (8u << 20)
int paraht_rht2ht_d_noalloc(paraht_ctx ctx, int n, double* A, int lda, double* B, int ldb, double* Q, int ldq,
                            double* Z, int ldz, int r, int nq, int flags);

/* ---- batched: `count` independent pencils of possibly different sizes (device pointers).
 * Arrays of length count; r, p, nq per pencil.  No counterpart in the reference (it reduces one
 * pencil per run).  Pencils with p*r <= 64 and n <= PARAHT_BATCH_MAX_N are reduced by one
 * persistent launch, one CTA per pencil at a time, largest first; their results are bitwise
 * those of paraht_reduce_d in FP64 (also when PARAHT_FLAG_SPLIT is set).  The other pencils go
 * through the single-pencil path, largest first, up to eight at a time on internal worker
 * contexts (own streams and workspace; their bulk lists on two side streams), overlapping the
 * persistent launch.  The worker contexts together use 32 streams: run with
 * CUDA_DEVICE_MAX_CONNECTIONS=32 (set before the process creates its CUDA context), or streams
 * share hardware queues and the pencils' kernels wait behind one another.
 * PARAHT_FLAG_BATCH_LOOP reduces the pencils one after the other with paraht_reduce_d on this
 * context (the looped baseline);
 * PARAHT_FLAG_GIVENS is refused (PARAHT_ERR_NOT_SUPPORTED).
 * Pointers of different pencils must not overlap. ---- */
#define PARAHT_BATCH_MAX_N 1024
#define PARAHT_FLAG_BATCH_LOOP 64
int paraht_reduce_batched_d(paraht_ctx ctx, int count, const int* n, double* const* A, const int* lda,
                            double* const* B, const int* ldb, double* const* Q, const int* ldq, double* const* Z,
                            const int* ldz, const int* r, const int* p, const int* nq, int flags);

/* ---- batch plans: the persistent batched launch as a replayable CUDA graph.  No counterpart in
 * the reference.  For a fixed set of pencils (device pointers, sizes and parameters as for
 * paraht_reduce_batched_d) reduced again and again with new values in the same arrays:
 * paraht_batch_plan_create checks them, groups them into buckets of equal (r, p, nq) (the
 * autotuner's per-size choice; each bucket gets its own shared-memory size and workspace),
 * uploads each bucket's pencil table once and captures the launches (per bucket: queue reset and
 * one persistent launch, the buckets on parallel branches) into a CUDA graph.
 * paraht_batch_plan_launch replays it on `stream` (cudaStream_t as void*, NULL: the legacy
 * default stream) and returns at once; synchronise the stream before reading the results.
 * Results are bitwise those of paraht_reduce_d in FP64.  Every pencil must be one the persistent
 * kernel takes (p r <= 64, n <= PARAHT_BATCH_MAX_N) and flags must be 0, else
 * PARAHT_ERR_NOT_SUPPORTED; -3 flags an invalid pencil, -16 a null plan pointer.  The plan holds
 * its own device buffers until paraht_batch_plan_destroy; replays of one plan must not overlap. ---- */
typedef struct paraht_batch_plan_s* paraht_batch_plan;
int paraht_batch_plan_create(paraht_ctx ctx, int count, const int* n, double* const* A, const int* lda,
                             double* const* B, const int* ldb, double* const* Q, const int* ldq, double* const* Z,
                             const int* ldz, const int* r, const int* p, const int* nq, int flags,
                             paraht_batch_plan* plan);
int paraht_batch_plan_launch(paraht_batch_plan plan, void* stream);
int paraht_batch_plan_destroy(paraht_batch_plan plan);

/* ---- LAPACK DGGHD3-compatible entry (no counterpart in the reference, which ignores ilo/ihi;
 * the argument list of dgghd3 as the reference driver calls it, src/profilereduction.f90:156,
 * without the work array): reduces rows/columns ilo..ihi (1-based) of the pencil, A and B
 * assumed upper triangular outside them as after balancing, by the two-stage reduction with
 * (r, p, nq), and applies the transformations to the rest of A and B.
 * compq/compz: 'N' Q/Z not referenced, 'I' Q/Z set to the identity first, 'V' Q/Z right-multiplied
 * (accumulated, as the reference does).  Status: LAPACK-style -i for the i-th argument
 * (1 compq .. 13 ldz, 14 r, 15 p, 16 nq), else as paraht_reduce_d.  _d: device pointers on ctx;
 * the plain form takes host arrays. ---- */
int paraht_gghd3_d(paraht_ctx ctx, char compq, char compz, int n, int ilo, int ihi, double* A, int lda, double* B,
                   int ldb, double* Q, int ldq, double* Z, int ldz, int r, int p, int nq, int flags);
int paraht_gghd3(char compq, char compz, int n, int ilo, int ihi, double* A, int lda, double* B, int ldb, double* Q,
                 int ldq, double* Z, int ldz, int r, int p, int nq, int flags);

/* ---- generalized eigenvalues of Hessenberg-triangular pencils: the QZ iteration that consumes
 * the reduced pencil (LAPACK DHGEQZ with JOB='E', COMPQ=COMPZ='N'; no counterpart in the
 * reference, whose driver stops at the reduced pencil, src/profilereduction.f90:156).
 * For i < count: H[i] (n[i] x n[i], leading dimension ldh[i]) upper Hessenberg and T[i] (ldt[i])
 * upper triangular, read only (entries below the structure are ignored).  Eigenvalue j of pencil
 * i is (alphar[i][j] + i alphai[i][j]) / beta[i][j] with beta >= 0, at its position j on the
 * diagonal of the final quasi-triangular pencil (as DHGEQZ orders them); beta = 0 marks an
 * infinite eigenvalue (T singular).  Real double-shift QZ
 * (Moler-Stewart, as DHGEQZ), a warp per pencil below n = 128 and a 2-warp CTA from there: real
 * eigenvalues have alphai exactly 0, complex ones come as adjacent exact conjugate pairs
 * (positive imaginary part first).  A diagonal entry of T at most eps ||T||_F counts as zero.
 * info[i] (host array): 0, or 2 when 30 n[i] sweeps did not converge (that pencil's outputs are
 * then incomplete).  _d: host arrays of device pointers, run on the context's stream and
 * synchronised; the plain form takes host arrays on this thread's default context.  Status: 0;
 * -2 count < 0, -3 an n < 0 (or null n), -4 .. -10 a null pointer among H, ldh, T, ldt, alphar,
 * alphai, beta (ldh, ldt: or below max(1, n)), -11 null info; else a PARAHT_ERR_ code (both
 * forms). ---- */
int paraht_hgeqz_eigs_d(paraht_ctx ctx, int count, const int* n, const double* const* H, const int* ldh,
                        const double* const* T, const int* ldt, double* const* alphar, double* const* alphai,
                        double* const* beta, int* info);
int paraht_hgeqz_eigs(int count, const int* n, const double* const* H, const int* ldh, const double* const* T,
                      const int* ldt, double* const* alphar, double* const* alphai, double* const* beta, int* info);

/* ---- failure-path self-test (no counterpart in the reference) ----
 * Runs the pipelined chase's bounded device-side wait on a progress word that nothing sets, with
 * a limit of spin_limit polls (1 .. 2^20, about 1 us each).  Returns the status the kernel
 * reported: PARAHT_ERR_TIMEOUT when the wait gave up as designed (the context stays usable),
 * 0 if it did not, PARAHT_ERR_CUDA on a launch failure, -2 for an invalid spin_limit. */
int paraht_selftest_wait_timeout(paraht_ctx ctx, long long spin_limit);
/* Self-test of the branch-free reflector scalars the generation chains use (DLARFG's tau, scal =
 * 1/(alpha - beta), beta from alpha and the squared norm of the reflector's tail): for i < count,
 * out[3i..3i+2] = tau, scal, beta of (alpha[i], xnorm2[i]); device pointers, stream-ordered on the
 * context's stream and synchronised.  -2 for count < 0, -3 for a null pointer. */
int paraht_selftest_reflector(paraht_ctx ctx, int count, const double* alpha, const double* xnorm2, double* out);

/* ---- misc ---- */
const char* paraht_strerror(int status);
int paraht_version(void);

#ifdef __cplusplus
}
#endif
#endif /* PARAHT_H */
