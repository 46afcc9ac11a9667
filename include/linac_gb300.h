/*
 * linac_gb300 -- C ABI of the GB300 (sm_103a) dense RREF / monomial-loader
 * library.
 *
 * Plain pointers and sizes only.  Every function returns an LNC_* status
 * (0 = success); on failure lnc_last_error() returns a message for the calling
 * thread.  Matrices are row-major with an explicit leading dimension counted
 * in elements.  dtype codes: LNC_U32 / LNC_U64 residues mod p, LNC_F64 reals,
 * LNC_C128 complex (interleaved real, imaginary doubles).
 *
 * The reference (GDeLaurentis/linac v1.0.1) exposes Python functions backed by
 * pycuda, not a C ABI; each entry point below names the reference interface it
 * replaces.  The library keeps per-device state (streams, cached device
 * properties, the no-allocation scratch address) for the life of the process;
 * none of it survives cudaDeviceReset.
 */
#ifndef LINAC_GB300_H
#define LINAC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define LNC_OK 0
#define LNC_ERR_INVALID (-1)   /* bad argument, shape or dtype              */
#define LNC_ERR_NOT_PRIME (-2) /* modulus is not prime (no inverse exists)  */
#define LNC_ERR_CUDA (-3)      /* CUDA runtime error (message has details)  */
#define LNC_ERR_OOM (-4)       /* device allocation failed                  */
#define LNC_ERR_TIMEOUT (-5)   /* a bounded device-side wait ran out        */
#define LNC_ERR_ADMISSION (-6) /* request rejected by memory admission      */
#define LNC_ERR_NO_DEVICE (-7) /* no CUDA device                            */
#define LNC_ERR_UNSUPPORTED (-8) /* valid request this build cannot serve   */

/* ---- element types ------------------------------------------------------ */
#define LNC_U32 1
#define LNC_U64 2
#define LNC_F64 3
#define LNC_C128 4

/* ---- flags for the RREF entry points ----------------------------------- */
#define LNC_FLAG_NONE 0
#define LNC_FLAG_NO_SCALING 1   /* float path: skip the row pre-scaling     */
#define LNC_FLAG_SIMT_TRAILING 2 /* force the SIMT trailing update (tests)  */
#define LNC_FLAG_ROBUST_PANEL 4  /* F_p: always use the exhaustive grid-wide panel */
/* F_p, 32-bit: do not redo a candidate panel that missed a pivot in place (no
 * grid-wide panel launch per panel, so concurrent solves on other streams are
 * never held up).  A miss is reported through dev_rank = -1 instead (the
 * outputs are then invalid and the caller redoes the solve with
 * LNC_FLAG_ROBUST_PANEL); a device-side timeout through dev_rank = -2.       */
#define LNC_FLAG_DEFER_FALLBACK 8
/* float64 / complex128: mixed precision.  Trailing updates run on the tensor
 * cores as exact products of 31-bit fixed-point operands (BF16 digits, FP32
 * accumulation); panels, pivot choice and threshold stay FP64; the non-pivot
 * columns of the result are then refined in FP64 (residual of the row-scaled
 * input, correction through the stored panel transforms) until the
 * correction stops shrinking.  When a pivot candidate's magnitude falls
 * between 10^-3 and 10^5 times the threshold (a rank decision the
 * reduced-precision updates could change) the solve is redone in FP64.  Synchronises the
 * stream; lnc_mixed_report describes the last such solve of the thread.     */
#define LNC_FLAG_MIXED 16
/* F_p: no look-ahead.  By default a large solve (>= 2^22 entries, at least
 * three panels) runs the next candidate panel on a second, high-priority
 * stream while the caller's stream applies the current panel to the columns
 * beyond it (fork and join through events, so stream capture records both);
 * this flag keeps every launch on the caller's stream (tests, timing).      */
#define LNC_FLAG_NO_LOOKAHEAD 32
/* F_p: look ahead at any shape with at least three panels (tests).         */
#define LNC_FLAG_LOOKAHEAD 64

/* ---- library / device ---------------------------------------------------- */
/* Version string of the library. */
const char* lnc_version(void);
/* Message of the last failed call on this thread ("" if none). */
const char* lnc_last_error(void);
/* Number of visible CUDA devices (0 when none).  Replaces the pycuda probe
 * behind CUDA_FOUND (linac/_optional.py:11-23). */
int lnc_device_count(void);
/* Select the device used by this thread's subsequent calls. */
int lnc_set_device(int device);
/* SM count, free and total device memory of the current device. */
int lnc_device_info(int* sms, size_t* free_bytes, size_t* total_bytes);
/* Number of kernels this library has launched (monotonic counter). */
int64_t lnc_launch_count(void);

/* ---- memory, streams, events (thin CUDA runtime wrappers, so that callers
 *      need no CUDA bindings of their own) ------------------------------------ */
int lnc_malloc(void** dev_ptr, size_t bytes);
int lnc_free(void* dev_ptr);
int lnc_malloc_host(void** host_ptr, size_t bytes); /* pinned host memory */
int lnc_free_host(void* host_ptr);
int lnc_memcpy_h2d(void* dst, const void* src, size_t bytes, void* stream);
int lnc_memcpy_d2h(void* dst, const void* src, size_t bytes, void* stream);
int lnc_memcpy_d2d(void* dst, const void* src, size_t bytes, void* stream);
int lnc_memset(void* dev_ptr, int value, size_t bytes, void* stream);
int lnc_stream_create(void** stream);
int lnc_stream_destroy(void* stream);
int lnc_stream_synchronize(void* stream);
int lnc_device_synchronize(void);
int lnc_event_create(void** event);
int lnc_event_destroy(void* event);
int lnc_event_record(void* event, void* stream);
int lnc_event_elapsed_ms(void* start, void* stop, float* ms);
/* Later work on `stream` waits for `event` (recorded on another stream). */
int lnc_stream_wait_event(void* stream, void* event);
/* Read (and clear) the device-side error word; returns the status it held
 * (LNC_OK when none): LNC_ERR_TIMEOUT from a bounded wait that ran out,
 * LNC_ERR_INVALID from lnc_load_matrix_device given an index past the end of
 * a bases row.  Synchronises the device. */
int lnc_device_status(void);

/* ---- kernel timing (CUDA events on the launching stream) ------------------ */
/* kernel classes: 0 panel, 1 trailing update, 2 loader, 3 gather, 4 batch */
int lnc_kernel_timing_enable(int enable);
int lnc_kernel_timing_reset(void);
/* Total launches and summed event time (ms) of one class since the reset;
 * synchronises the events it reads. */
int lnc_kernel_timing_read(int kernel_class, int64_t* launches, double* total_ms);
/* Algorithmic work of the timed launches of one class since the reset:
 * field multiply-adds (trailing update, nominal contraction depth 128 per
 * panel), bytes moved (panel, loader, gather). */
int lnc_kernel_timing_work(int kernel_class, double* work);

/* ---- RREF ------------------------------------------------------------------ */
/*
 * Reduced row-echelon form of a host matrix: reads host_in (m x n, leading
 * dimension ld_in elements), writes the RREF to host_out (ld_out; may equal
 * host_in).  p is the field characteristic (ignored for LNC_F64 / LNC_C128,
 * where `tol` is the head threshold and the rows are pre-scaled by their
 * largest |a| unless LNC_FLAG_NO_SCALING).  Optional outputs: pivot_cols
 * (min(m,n) entries, -1 past the rank) and *rank.  Synchronous.
 * Replaces cuda_row_reduce (linac/pycuda_row_reduce.py:18-151): the H2D copy
 * (:71-79), the per-column launch loop (:94-131) and the D2H copy (:141-149).
 */
int lnc_rref_host(int dtype, int64_t m, int64_t n, uint64_t p, double tol, const void* host_in,
                  int64_t ld_in, void* host_out, int64_t ld_out, int64_t* pivot_cols, int64_t* rank,
                  int flags);

/*
 * Device-resident RREF on `stream`.  `dev_work` (m x n, ld_work) holds the
 * input and is destroyed; the RREF is written to `dev_out` (ld_out), which may
 * equal dev_work.  dev_pivot_cols (min(m,n) int64) and dev_rank (one int64)
 * are optional device outputs.  Asynchronous: errors of bounded device waits
 * surface through lnc_device_status().
 * Replaces the device half of cuda_row_reduce (linac/pycuda_row_reduce.py:81-131)
 * and its kernels (linac/row_reduce.cu:117-430).
 */
int lnc_rref_device(int dtype, int64_t m, int64_t n, uint64_t p, double tol, void* dev_work,
                    int64_t ld_work, void* dev_out, int64_t ld_out, int64_t* dev_pivot_cols,
                    int64_t* dev_rank, void* stream, int flags);

/*
 * The same device RREF as lnc_rref_device, but allocating nothing: its scratch
 * is a fixed 16 MiB array in the library's device memory instead of
 * stream-ordered allocations.  For callers that cannot allocate device memory
 * when they need the result -- a host framework that reserved all of HBM for
 * its own pool up front, or a latency-critical thread that must not wait on an
 * allocator.  No counterpart in the reference (linac always allocates through
 * pycuda).  Limits: dev_out must not overlap dev_work at all; sizes whose
 * scratch exceeds 16 MiB (about m + n > 30,000 for uint32 residues) are
 * rejected with LNC_ERR_INVALID.  The first call on a device looks up the
 * array's device address (make it before any stream capture) and keeps it
 * for the life of the process (it does not survive cudaDeviceReset); all
 * calls share the array, so calls that overlap on the GPU race.
 */
int lnc_rref_device_noalloc(int dtype, int64_t m, int64_t n, uint64_t p, double tol, void* dev_work,
                            int64_t ld_work, void* dev_out, int64_t ld_out, int64_t* dev_pivot_cols,
                            int64_t* dev_rank, void* stream, int flags);

/* ---- batched RREF (many uneven matrices, a prime each) ---------------------- */
typedef struct lnc_batch_matrix {
    uint64_t p;             /* prime: < 2^32 for LNC_U32, any for LNC_U64, ignored for floats */
    int64_t m, n;
    const void* dev_in;     /* m x n input (not modified), leading dimension ld_in */
    int64_t ld_in;
    void* dev_out;          /* m x n RREF, leading dimension ld_out */
    int64_t ld_out;
    int64_t* dev_pivot_cols; /* optional: min(m,n) pivot columns, -1 past the rank */
    int64_t* dev_rank;       /* optional */
} lnc_batch_matrix;

/*
 * Plan a batched RREF of `count` matrices (LNC_U32 only): allocates one
 * scratch arena, records every launch of every panel step and captures them
 * into one CUDA graph.  tiles_per_cta / cand_rows tune the contraction work
 * split and the candidate-block height (0 = defaults).  The plan can be run
 * any number of times on new contents of the same buffers.
 * No counterpart in the reference: linac reduces one matrix per
 * cuda_row_reduce call (linac/pycuda_row_reduce.py:18-151); its callers loop
 * (linac/vector_spaces/over_function_fields.py:74-101).
 */
int lnc_batch_plan_create(int dtype, const lnc_batch_matrix* mats, int64_t count, int tiles_per_cta,
                          int cand_rows, void* stream, void** plan);
/* One graph launch on `stream` (asynchronous). */
int lnc_batch_plan_run(void* plan, void* stream);
/* Synchronise; redo any matrix whose candidate panels missed a pivot with the
 * exhaustive path; *n_redo (optional) receives how many. */
int lnc_batch_plan_finish(void* plan, void* stream, int64_t* n_redo);
/* Device bytes held by the plan (admission accounting). */
int64_t lnc_batch_plan_bytes(void* plan);
/* One CUDA graph over `count` plans (a batch cut into chunks): each plan's
 * graph is a child graph, with no dependency between plans, so one launch
 * (lnc_batch_group_run, asynchronous) reduces every chunk and the GPU
 * overlaps them.  The plans must outlive the group and must not run on their
 * own while a group run is in flight; once the group's stream has completed
 * the run (synchronise it, or make each plan's stream wait on it),
 * lnc_batch_plan_finish of each plan completes the run.  No counterpart in the
 * reference (see lnc_batch_plan_create). */
int lnc_batch_group_create(void* const* plans, int64_t count, void** group);
int lnc_batch_group_run(void* group, void* stream);
int lnc_batch_group_destroy(void* group);
int lnc_batch_plan_destroy(void* plan);
/* LNC_U32: create + run + finish + destroy.  LNC_U64 (a prime per matrix, up
 * to 2^64 - 59; no captured plan): every matrix through the single-matrix
 * 64-bit path, on 16 worker threads with their own streams, after the work
 * already queued on `stream`; synchronous.  Inputs are not modified. */
int lnc_rref_batch_device(int dtype, const lnc_batch_matrix* mats, int64_t count, void* stream, int flags);

/* ---- batched float / complex RREF --------------------------------------------- */
typedef struct lnc_mixed_result {
    int iterations;        /* refinement iterations (LNC_FLAG_MIXED)                   */
    int redone_fp64;       /* 1: a rank decision was close, the solve was redone in FP64 */
    double error_estimate; /* as lnc_mixed_error_estimate; 0 without LNC_FLAG_MIXED     */
} lnc_mixed_result;

/*
 * RREF of `count` float64 / complex128 matrices of any sizes (LNC_F64 or
 * LNC_C128; `p` of each descriptor is ignored), `tol` the head threshold
 * (<= 0: 1e-9), flags as for lnc_rref_device (LNC_FLAG_MIXED for the
 * mixed-precision path).  `workers` host threads (<= 0: 16), each with its own
 * stream, take the matrices in order and solve them concurrently; inputs are
 * not modified.  reports (optional, count entries) receives each solve's
 * mixed-precision report.  Synchronous.
 * No counterpart in the reference: linac reduces one matrix per
 * cuda_row_reduce call (linac/pycuda_row_reduce.py:18-151).
 */
int lnc_rref_float_batch(int dtype, const lnc_batch_matrix* mats, int64_t count, double tol, int flags,
                         int workers, lnc_mixed_result* reports);

/* ---- workload helpers (no counterpart in the reference) --------------------- */
/* Fill `count` residues uniform in [0, p) from `seed` (LNC_U32 / LNC_U64). */
int lnc_fill_uniform_modp(void* dev_ptr, int64_t count, uint64_t p, uint64_t seed, int dtype, void* stream);
/* C = A B mod p, A m x k, B k x n, exact: LNC_U32 (p < 2^32) on the
 * tensor-core limb GEMM, LNC_U64 (odd p) on a SIMT Montgomery kernel.  Used
 * to build rank-deficient inputs B.C on the device and to certify the RREF
 * [I | X] of an augmented system [A | B] (A X = B mod p). */
int lnc_matmul_modp_device(int dtype, int64_t m, int64_t k, int64_t n, uint64_t p, const void* A, int64_t lda,
                           const void* B, int64_t ldb, void* C, int64_t ldc, void* stream);

/* Outcome of the calling thread's last LNC_FLAG_MIXED solve: refinement
 * iterations, the last correction's max-norm relative to the refined
 * entries, and whether the solve was redone in FP64.  No reference
 * counterpart (linac's float path is FP64 only, linac/row_reduce.cu:55-270). */
int lnc_mixed_report(int* iterations, double* last_correction, int* redone_fp64);
/* Error estimate of the calling thread's last LNC_FLAG_MIXED solve: the
 * max-norm of one further refinement correction (FP64 residual of the result
 * through the stored panel transforms, computed and not applied) relative to
 * the largest refined entry -- an a-posteriori estimate of the result's
 * max-norm error against the exact RREF of the row-scaled input.  0 when no
 * entry needed refinement (full column rank: the result is exact), -1 when
 * the solve was redone in FP64.  No reference counterpart. */
int lnc_mixed_error_estimate(double* error_estimate);

/* ---- incremental RREF --------------------------------------------------------- */
/*
 * RREF of [rows so far; k new rows] from the RREF of the rows so far, over F_p
 * with 32-bit residues.  dev_rref (r x n, ld_rref) holds the r non-zero RREF
 * rows with pivot columns dev_pivot_cols[0..r) (increasing) and is
 * overwritten with those rows cleared in the new pivot columns; dev_new is
 * k x n (ld_new, residues); dev_out ((r + k) x n, ld_out) receives the RREF of
 * the stacked rows, zero rows after the rank; its pivot columns and rank go to
 * dev_out_pivot_cols (r + k entries) and dev_out_rank.  Costs k r n + r s n
 * multiply-adds (s new pivots) plus a k-row RREF; synchronises the stream
 * once.  No reference counterpart: linac re-reduces the grown matrix from
 * scratch (linac/vector_spaces/over_function_fields.py:74-101).
 */
int lnc_rref_append_device(int dtype, int64_t r, int64_t k, int64_t n, uint64_t p, void* dev_rref,
                           int64_t ld_rref, const int64_t* dev_pivot_cols, const void* dev_new,
                           int64_t ld_new, void* dev_out, int64_t ld_out, int64_t* dev_out_pivot_cols,
                           int64_t* dev_out_rank, void* stream);

/* ---- null space ------------------------------------------------------------- */
/*
 * Canonical null-space basis of an RREF R (r x n, ld_rref, device) with pivot
 * columns dev_pivot_cols[0..r) (increasing): out (n x (n - r), ld_out, device,
 * R's element type) with out[Pc[t], j] = R[t, Nc[j]] and out[Nc[i], j] =
 * -[i == j] (-1 is p - 1 over F_p; p = 2^32 for uint32 or 0 for uint64 writes
 * the all-ones word, a marker no residue equals), Nc the non-pivot columns in
 * order.
 * Replaces canonical_kernel_from_row_reduced_echelon_form
 * (linac/linear_algebra_tools.py:54-63), which runs on the host.
 */
int lnc_canonical_kernel_device(int dtype, int64_t r, int64_t n, uint64_t p, const void* dev_rref,
                                int64_t ld_rref, const int64_t* dev_pivot_cols, void* dev_out,
                                int64_t ld_out, void* stream);

/* ---- monomial loader --------------------------------------------------------- */
/*
 * out[r, c] = prod_{t<degree} bases[r, lindices[c, t]] (mod p for LNC_U32 /
 * LNC_U64; plain products for LNC_F64 / LNC_C128), folded left to right; a
 * single factor is copied as is.  bases is n_rows x basis_len, lindices is
 * n_cols x degree (uint32), out is n_rows x n_cols (ld_out).  An index >=
 * basis_len is an error: the host entry returns LNC_ERR_INVALID before any
 * device work; the device entry (which cannot read the indices on the host)
 * writes 0 to the affected columns and raises the device error word to
 * LNC_ERR_INVALID (lnc_device_status).
 * Replaces cuda_load_matrix (linac/pycuda_matrix_loader.py:27-124) and its
 * kernel LoadMatrix (linac/matrix_loader.cu:88-112).
 */
int lnc_load_matrix_host(int dtype, int64_t n_rows, int64_t n_cols, int64_t basis_len,
                         int64_t degree, uint64_t p, const void* host_bases,
                         const uint32_t* host_lindices, void* host_out);
int lnc_load_matrix_device(int dtype, int64_t n_rows, int64_t n_cols, int64_t basis_len,
                           int64_t degree, uint64_t p, const void* dev_bases,
                           const uint32_t* dev_lindices, void* dev_out, int64_t ld_out,
                           void* stream);

/* ---- serving loop ------------------------------------------------------------ */
/*
 * A server owns a scheduler thread and a set of CUDA streams ("slots").
 * Requests (an RREF of a host matrix, or a monomial load followed by the RREF
 * of the loaded matrix) are queued by lnc_serve_submit and admitted while a
 * slot is free and their device footprint (lnc_serve_request_bytes) fits the
 * memory budget; an admitted request's matrix stays resident on the device
 * from its load to its result copy, and the requests in flight run
 * concurrently on their streams.  Requests that arrive while others run are
 * admitted as slots and memory free up (continuous batching; later requests
 * may pass a queued one that does not fit yet, a bounded number of times).
 * F_p solves run with LNC_FLAG_DEFER_FALLBACK; a solve whose candidate panels
 * missed a pivot is redone with LNC_FLAG_ROBUST_PANEL before it completes.
 *
 * Host buffers must stay valid until the request completes; page-locked
 * buffers (lnc_malloc_host) let the copies overlap, pageable ones make the
 * scheduler wait for each copy.
 *
 * No reference counterpart: linac's callers make one synchronous
 * cuda_row_reduce / load_matrices call per system
 * (linac/pycuda_row_reduce.py:18-151, linac/pycuda_matrix_loader.py:127-230).
 */
#define LNC_SERVE_RREF 1      /* RREF of host_in (m x n, ld_in)                       */
#define LNC_SERVE_LOAD_RREF 2 /* load (bases, lindices) into an m x n matrix, then RREF */

typedef struct lnc_serve_request {
    int kind;                       /* LNC_SERVE_RREF or LNC_SERVE_LOAD_RREF          */
    int dtype;                      /* LNC_U32 / LNC_U64 / LNC_F64 / LNC_C128          */
    uint64_t p;                     /* prime (F_p dtypes)                              */
    double tol;                     /* pivot threshold (float dtypes; <= 0: 1e-9)      */
    int64_t m, n;                   /* matrix shape (load: points x monomials)         */
    const void* host_in;            /* RREF: input matrix                              */
    int64_t ld_in;
    const void* host_bases;         /* load: m x basis_len values (dtype)              */
    int64_t basis_len;
    const uint32_t* host_lindices;  /* load: n x degree basis indices                  */
    int64_t degree;
    void* host_out;                 /* m x n result (ld_out)                           */
    int64_t ld_out;
    int64_t* host_pivot_cols;       /* min(m, n) entries (first rank valid) or NULL    */
    int64_t* host_rank;             /* or NULL                                         */
    int flags;                      /* LNC_FLAG_* for the solve                        */
} lnc_serve_request;

typedef struct lnc_serve_stats {
    int64_t submitted, completed, failed, redone;
    int64_t queued, inflight;
    int64_t bytes_in_use, peak_bytes, budget_bytes;
    double p50_ms, p99_ms, mean_ms, max_ms; /* submit -> result on the host, completed requests */
} lnc_serve_stats;

/* budget_bytes <= 0: 90% of the device memory free at creation; max_inflight <= 0: 16 */
int lnc_server_create(int64_t budget_bytes, int max_inflight, void** server);
/* cancels queued requests (LNC_ERR_INVALID), waits for those in flight */
int lnc_server_destroy(void* server);
/* device bytes the request holds while in flight (its admission size) */
int64_t lnc_serve_request_bytes(const lnc_serve_request* req);
/* LNC_ERR_ADMISSION when the request alone exceeds the budget */
int lnc_serve_submit(void* server, const lnc_serve_request* req, int64_t* ticket);
/* done = 1 once the results are in the host buffers; status = the request's LNC_* code */
int lnc_serve_poll(void* server, int64_t ticket, int* done, int* status);
/* LNC_OK when the request completed within timeout_s (< 0: no limit), else LNC_ERR_TIMEOUT */
int lnc_serve_wait(void* server, int64_t ticket, double timeout_s, int* status);
/* queue_ms: submit -> admission; total_ms: submit -> results on the host */
int lnc_serve_latency(void* server, int64_t ticket, double* queue_ms, double* total_ms);
/* forget a completed ticket */
int lnc_serve_release(void* server, int64_t ticket);
int lnc_serve_stats_read(void* server, lnc_serve_stats* out);
int lnc_serve_stats_reset(void* server);

#ifdef __cplusplus
}
#endif

#endif /* LINAC_GB300_H */
