/*
 * rqsqd.h -- C ABI of the GB300 (sm_103a) SQD hot path: the Pauli-sum matvec restricted to a
 * sorted bitstring subspace, and the single-vector LOBPCG that drives it.
 *
 * Reference interfaces replaced (rqutils 0.2.0, pure JAX, no FFI of its own):
 *   rq_subspace_build      uniquify_states / the sort inside get_xsource   rqutils/sqd.py:414-503
 *   rq_xsource             get_xsource                                   rqutils/sqd.py:448-503
 *   rq_diagonal            get_diagonal                                  rqutils/sqd.py:554-575
 *   rq_conn_build          the cached X-source table (cache_level[0]==1) rqutils/sqd.py:318-326
 *   rq_matvec              apply_h / apply_h_x_cached / apply_h_xz_cached rqutils/sqd.py:590-684
 *   rq_fullspace_matvec    PauliSumXZ.matmul                             rqutils/paulis/symplectic.py:131-150
 *   rq_lobpcg_solve        ground_locg / _ground_locg_callable            rqutils/ground_locg.py:128-377
 *   rq_lobpcg_solve_cb     ground_locg with a user matvec or matrix      rqutils/ground_locg.py:154-179
 *   rq_eigenpair_3x3       eigenpair_3x3                                 rqutils/ground_locg.py:438-471
 *   rq_batch_*             sqd() over many problems (no batched form in the reference; each
 *                          problem is the reference's sqd.py:299-411 / ground_locg.py:182-377)
 *
 * Conventions
 *   - A basis state is a uint64 whose bit q is qubit q.  Subspaces are strictly increasing arrays
 *     of such states (the reference's lexicographic order of packed bytes is the same order).
 *   - A Hamiltonian is grouped by X signature: group j has X mask xmask[j] and terms
 *     toff[j] <= k < toff[j+1] with Z mask zmask[k] and phased coefficient coef[2k] + i coef[2k+1]
 *     (the coefficient times (-i)^popcount(x & z)).  Within a group the terms end at the first
 *     zero coefficient, as in the reference's diagonal loop.
 *   - (H v)[i] = sum_j sum_k c_jk (-1)^popcount(S[i] & z_jk) v[m],  S[m] = S[i] ^ x_j;
 *     a term whose source S[i] ^ x_j is not in the subspace contributes nothing.
 *   - Every pointer inside the structs below is a DEVICE pointer owned by the caller.  No entry
 *     point allocates device memory; workspaces are sized by the *_size functions and passed in.
 *   - Every call is ordered on the given stream (cudaStream_t passed as void*; NULL = legacy
 *     default stream).  Calls that return a host-visible result synchronise that stream.
 *   - Return value: RQ_OK (0) or an RQ_E* code; rq_last_error() gives a message (thread-local).
 *   - Not thread-safe per workspace: concurrent calls must use distinct workspaces.
 */
#ifndef RQSQD_H
#define RQSQD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* value types of vectors */
#define RQ_F32  0   /* float                       */
#define RQ_F64  1   /* double                      */
#define RQ_C64  2   /* complex float  (re, im)     */
#define RQ_C128 3   /* complex double (re, im)     */

/* status codes */
#define RQ_OK            0
#define RQ_E_ARG         1   /* invalid argument / size                                   */
#define RQ_E_CUDA        2   /* CUDA runtime error                                        */
#define RQ_E_UNSORTED    3   /* subspace not strictly increasing                          */
#define RQ_E_TABLE       4   /* hash table overflow (bounded probe or insert gave up)     */
#define RQ_E_NONFINITE   5   /* a non-finite value appeared (LOBPCG breakdown)            */
#define RQ_E_MAXITER     6   /* LOBPCG stopped at maxiter without meeting the tolerance   */
#define RQ_E_RANGE       7   /* a size exceeds a fixed limit of the entry point           */

/* lookup structures for S[i] ^ x membership */
#define RQ_LOOKUP_HASH     0  /* open addressing, buckets of 4 keys (uint32 or uint64)         */
#define RQ_LOOKUP_BSEARCH  1  /* shared-memory sampled binary search over the sorted states      */
#define RQ_LOOKUP_IDENTITY 2  /* full space: S[i] = i, D = 2^n (PauliSumXZ.matmul)               */

/* matvec modes (the reference's cache_level) */
#define RQ_MODE_FREE 0   /* cache_level (0, *): lookups inside every matvec                        */
#define RQ_MODE_CONN 1   /* cache_level (1, 0|1): connectivity cached, diagonals recomputed        */
#define RQ_MODE_CSR  2   /* cache_level (*, 2): full CSR of matrix elements                        */

#define RQ_FILTER_WORDS 133  /* 65 x 65 bitset of (popcount(s & fmask_a), popcount(s & fmask_b)) */

typedef struct rq_subspace {
    const uint64_t *states;  /* [D] strictly increasing                                   */
    int64_t   D;             /* subspace dimension, 1 <= D < 2^31                          */
    void     *hkeys;         /* 2^hbits buckets of 4 keys: (key_bits / 2) << hbits bytes,
                                16-byte aligned                                            */
    int32_t  *hvals;         /* [4 << hbits] row index of each key slot, 16-byte aligned   */
    int32_t   hbits;         /* log2(number of buckets), from rq_subspace_sizes            */
    int32_t   lookup;        /* RQ_LOOKUP_*                                                */
    int32_t   key_bits;      /* 32: states and every X mask < 2^32 (16-byte buckets); 64   */
    int32_t   pbits;         /* presence bitmap size log2 (rq_presence_bits), 0 = none     */
    uint64_t  empty_key;     /* written by rq_subspace_build: a value not in states        */
    uint64_t  fmask_a;       /* sector filter masks (0, 0 = filter off)                    */
    uint64_t  fmask_b;
    uint32_t *fbits;         /* [RQ_FILTER_WORDS], written by rq_subspace_build            */
    uint32_t *pmap;          /* [2^pbits / 32]: bit (hash(s) >> (32 - pbits)) set for every
                                state, written by rq_subspace_build; a lookup whose bit is
                                clear skips the table (NULL = none)                        */
    uint32_t *lmap;          /* line filter, [2^lbits lines of 2^lwbits bits] or NULL: for
                                every state, with h = hash(s), bits h mod 32 and h >> 27 of word
                                (h mod 2^lwbits) >> 5 of line hash(s >> lshift) >> (32 -
                                lbits), written by rq_subspace_build.
                                States that agree above bit lshift share a line, and so do
                                their targets under one X mask: the rows of a warp (consecutive
                                sorted states) probe a few lines instead of one line per lane.
                                A clear bit is a miss; two set bits are resolved in the table */
    int32_t   lbits;         /* log2(lines) of lmap, from rq_line_filter_bits               */
    int32_t   lwbits;        /* log2(bits per line): 8 (32-byte lines) .. 10 (128-byte)     */
    int32_t   lshift;        /* written by rq_subspace_build: the prefix shift, chosen so that
                                about 2^(lwbits - 5) states share a prefix on average        */
    int32_t   fpoint;        /* written by rq_subspace_build: pa * 65 + pb when every state has
                                the same pair pa = popcount(s & fmask_a), pb = popcount(s &
                                fmask_b) (a subspace in one sector), else -1; -1 with the
                                filter off                                                  */
} rq_subspace_t;

typedef struct rq_terms {
    int32_t   J;             /* number of X groups                                         */
    int32_t   K;             /* number of terms (sum of group sizes)                       */
    int32_t   diag_group;    /* index of the group with x = 0, or -1                       */
    int32_t   is_real;       /* 1 if every coefficient is real (real vectors allowed)      */
    const uint64_t *xmask;   /* [J]                                                        */
    const int32_t  *toff;    /* [J + 1]                                                    */
    const uint64_t *zmask;   /* [K]                                                        */
    const double   *coef;    /* [2K] interleaved (re, im)                                  */
    const uint32_t *xhash;   /* [J] bucket hash of each X mask (rq_terms_hash), or NULL    */
} rq_terms_t;

typedef struct rq_operator {
    rq_subspace_t sub;
    rq_terms_t    terms;
    int32_t       mode;      /* RQ_MODE_*                                                  */
    int32_t       val_vtype; /* value type of `val` (RQ_MODE_CSR); a matvec of another type
                                converts on load                                           */
    const double *diag0;     /* [D] real diagonal of group diag_group, or NULL (computed)  */
    const int64_t *rowptr;   /* [D + 1]  RQ_MODE_CONN / RQ_MODE_CSR                        */
    const int32_t *col;      /* [nnz]    source row of each off-diagonal element           */
    const int32_t *grp;      /* [nnz]    X group of each element (RQ_MODE_CONN)            */
    const void    *val;      /* [nnz]    element values in the matvec's value type (CSR)   */
    int64_t       nnz;
} rq_operator_t;

/* ---- sizing (host only) ---------------------------------------------------------------- */

/* Hash-table bucket count exponent for D states at load factor <= 1/8 (4 keys per bucket):
 * hkeys takes (key_bits / 2) << hbits bytes, hvals 4 << hbits int32. */
int rq_subspace_sizes(int64_t D, int32_t key_bits, int32_t *hbits);

/* Presence bitmap size for D states: 0 when the hash table is small enough to stay in L2
 * (<= 64 MB), else pbits = min(29, hbits + 2) (at most 64 MB of bitmap, a bit set for ~1/8 of
 * the misses).  The bitmap takes 2^pbits / 8 bytes. */
int rq_presence_bits(int64_t D, int32_t key_bits, int32_t *pbits);

/* Line-filter size for D states and 2^lwbits bits per line (lwbits 8..10): 2^lbits lines, each
 * holding 2^(lwbits - 7) states on average (lbits at most 37 - lwbits, so that a word index fits
 * 32 bits: beyond 2^29 states the lines fill fuller); the filter takes 2^(lbits + lwbits - 3)
 * bytes. */
int rq_line_filter_bits(int64_t D, int32_t lwbits, int32_t *lbits);

/* Bytes of scratch that rq_matvec / rq_conn_build / rq_dots need for their reductions/scans. */
int rq_scratch_size(int64_t D, size_t *bytes);

/* ---- subspace ---------------------------------------------------------------------------- */

/* Validate strict increase, choose empty_key, fill the hash table and the sector filter.
 * Synchronises the stream; returns RQ_E_UNSORTED when states is not strictly increasing. */
int rq_subspace_build(rq_subspace_t *sub, void *scratch, void *stream);

/* get_xsource for J X masks: out[j * D + i] = m with S[m] = S[i] ^ xmask[j], else -1. */
int rq_xsource(const rq_subspace_t *sub, const uint64_t *xmask, int32_t J, int32_t *out,
               void *stream);

/* get_diagonal: out[i] = sum_k c_k (-1)^popcount(S[i] & z_k), k < K, stopping at the first
 * zero coefficient.  out is complex double [2D]. */
int rq_diagonal(const uint64_t *states, int64_t D, const uint64_t *zmask, const double *coef,
                int32_t K, double *out, void *stream);

/* Upload grouped terms from HOST arrays (X masks strictly increasing, group offsets toff[J+1]
 * from 0 to K, coefficients interleaved re/im) into caller-owned device buffers d_xmask[J],
 * d_toff[J+1], d_zmask[K], d_coef[2K], d_xhash[J]; fill *t (J, K, diag_group, is_real, the
 * device pointers) and compute the X hashes.  The device form of PauliSumXZ
 * (symplectic.py:42-49).  Synchronises the stream; the host arrays may be freed on return. */
int rq_terms_upload(int32_t J, int32_t K, const uint64_t *xmask, const int32_t *toff,
                    const uint64_t *zmask, const double *coef, uint64_t *d_xmask, int32_t *d_toff,
                    uint64_t *d_zmask, double *d_coef, uint32_t *d_xhash, rq_terms_t *t,
                    void *stream);

/* Fill xhash[j] with the lookup hash of xmask[j] (used by RQ_LOOKUP_HASH matvecs: a row's
 * target bucket is hash(row) ^ xhash[j]).  Setup call, stream-ordered. */
int rq_terms_hash(const rq_terms_t *terms, uint32_t *xhash, void *stream);

/* Scratch bytes of rq_terms_group for K input terms. */
int rq_terms_group_scratch_size(int64_t K, size_t *bytes);

/* PauliSumXZ.from_paulisum (rqutils/paulis/symplectic.py:58-125) on the device, for K terms
 * already parsed into DEVICE arrays xmask[K], zmask[K] (bit q = qubit q, n <= 64) and coef[2K]
 * (complex128 interleaved), in input order: drops exact-zero coefficients, merges equal strings
 * (coefficients added from 0 in input order, terms in the lexicographic order of their labels:
 * character 0 = qubit n-1, I < X < Y < Z), keeps the real parts when force_real, groups by X
 * mask in ascending order (members in label order) and multiplies each coefficient by
 * (-i)^(popcount(x & z) mod 4).  Output (device, sized for K): xmask_out[J], toff_out[J + 1]
 * (int64), zmask_out[K'], coef_out[2K'] (phased); *J_out, *K_out; *flags_out bit 0 = an imaginary
 * part was dropped under force_real (the reference warns), bit 1 = every phased coefficient is
 * real.  Synchronises the stream. */
int rq_terms_group(int64_t K, const uint64_t *xmask, const uint64_t *zmask, const double *coef,
                   int32_t force_real, uint64_t *xmask_out, int64_t *toff_out,
                   uint64_t *zmask_out, double *coef_out, int64_t *J_out, int64_t *K_out,
                   int32_t *flags_out, void *scratch, void *stream);

/* ---- sample front end ------------------------------------------------------------------ */

/* Pack the reference's (rows, n) 0/1 sample rows (uint8, row stride in bytes) into uint64
 * states, column 0 = qubit n-1 (the bit layout of sqd.py:237 without its padding bit). */
int rq_pack_states(const uint8_t *bits, int64_t rows, int32_t n, int64_t row_stride,
                   uint64_t *out, void *stream);

/* Sort n uint64 samples and drop duplicates (uniquify_states, sqd.py:414-445, without the fill
 * rows): out[0 .. *count) strictly increasing; `in` is left unchanged and must not alias out.
 * Device radix sort (digits on which every sample agrees are skipped).  Synchronises the
 * stream (the count is returned on the host). */
int rq_uniquify_scratch_size(int64_t n, size_t *bytes);
int rq_uniquify(const uint64_t *in, int64_t n, uint64_t *out, int64_t *count, void *scratch,
                void *stream);

/* ---- connectivity cache ---------------------------------------------------------------- */

/* Pass 1 (col == NULL): fill rowptr[D+1] and return nnz.  Pass 2: fill col / grp (and val in
 * value type vtype when val != NULL) in row order, groups ascending within a row. */
int rq_conn_build(const rq_operator_t *op, int64_t *rowptr, int32_t *col, int32_t *grp,
                  void *val, int32_t vtype, int64_t *nnz, void *scratch, void *stream);

/* ---- matvec -------------------------------------------------------------------------------- */

/* y = H x in value type vtype (RQ_F32 / RQ_F64 need terms.is_real).  x and y must not alias. */
int rq_matvec(const rq_operator_t *op, int32_t vtype, const void *x, void *y, void *scratch,
              void *stream);

/* Full-space matvec (PauliSumXZ.matmul): D = 2^n, n <= 31, no subspace. */
int rq_fullspace_matvec(const rq_terms_t *terms, int32_t n, int32_t vtype, const void *x,
                        void *y, void *stream);

/* ---- LOBPCG --------------------------------------------------------------------------------- */

#define RQ_LOBPCG_REFERENCE 0   /* four matvecs per iteration, as ground_locg.py:288-341      */
#define RQ_LOBPCG_FAST      1   /* one matvec per iteration (A x, A y carried by linearity)   */

typedef struct rq_lobpcg_params {
    int32_t maxiter;        /* per phase; reference default 1000                            */
    int32_t variant;        /* RQ_LOBPCG_*                                                   */
    int32_t vtype;          /* value type of the (final) phase: RQ_F64 or RQ_C128 (or 32-bit)*/
    int32_t mixed;          /* 1: iterate first in the 32-bit type, then refine in vtype      */
    double  tol;            /* <= 0: machine epsilon of vtype (reference default)            */
    double  tol_dim;        /* vector length in the convergence test (<= 0: D)               */
    double  switch_rel;     /* mixed: leave the 32-bit phase when |r| < switch_rel * |theta|  */
    double  target_rel;     /* > 0: also stop when |r| <= target_rel * |theta| (FP64 residual) */
    int32_t refresh;        /* FAST: recompute A x, A y every `refresh` iterations (0 = 32)  */
    int32_t use_graph;      /* 0: eager launches; 1: one persistent cooperative kernel per
                               precision phase for RQ_MODE_CONN / RQ_MODE_CSR operators, CUDA
                               graphs of 8 iterations otherwise; 2: CUDA graphs only; 3: the
                               persistent kernel where 1 would use it, eager launches
                               otherwise (no graph is ever instantiated)                    */
    int32_t jacobi;         /* 1: precondition the residual with (diag(H) - theta)^-1        */
    int32_t guard;          /* 1: where the reference arithmetic gives 0/0 (a degenerate
                               Cardano eigenvector, |s| = 0) take a finite replacement; only
                               results that would otherwise be NaN change                    */
    int32_t restart;        /* FAST, one problem: drop the search direction and restart the
                               step from x every `restart` iterations of a phase (0 = never;
                               the reference never restarts; < 0 is rejected with RQ_E_ARG)   */
    int32_t pad_;
} rq_lobpcg_params_t;

typedef struct rq_lobpcg_result {
    double  eigval;         /* lowest Rayleigh-Ritz value                                      */
    double  resnorm;        /* |A x - eigval x| in FP64 after the last iteration              */
    double  axnorm;         /* |A x|                                                          */
    int32_t niter;          /* loop iterations (all phases)                                   */
    int32_t niter_lo;       /* iterations of the 32-bit phase                                 */
    int32_t matvecs;        /* matvecs issued                                                 */
    int32_t converged;      /* reference convergence test met                                 */
    int32_t status;         /* RQ_OK / RQ_E_NONFINITE / RQ_E_MAXITER                          */
    int32_t pad_;
} rq_lobpcg_result_t;

/* Workspace bytes for rq_lobpcg_solve on D rows. */
int rq_lobpcg_workspace_size(int64_t D, const rq_lobpcg_params_t *prm, size_t *bytes);

/* Lowest eigenpair of H from the initial vector x0 (value type prm->vtype, length D); the
 * normalised eigenvector is written to x_out (same type).  Synchronises the stream. */
int rq_lobpcg_solve(const rq_operator_t *op, const rq_lobpcg_params_t *prm, void *workspace,
                    const void *x0, void *x_out, rq_lobpcg_result_t *res, void *stream);

/* rq_lobpcg_solve without a caller workspace: no counterpart in the reference.  For callers
 * that cannot allocate device memory: a custom-call handler inside another framework gets only
 * its operand and result buffers (that framework's pool allocator owns the rest of the device
 * memory), and a service that reserves its device memory at start-up cannot let a library
 * cudaMalloc fail or fragment that reserve later.  The workspace is a static 8 MiB device array
 * of the library, held on every GPU that loads it until the process exits; problems whose
 * rq_lobpcg_workspace_size exceeds 8 MiB are rejected with RQ_E_RANGE (about 60,000 rows in
 * complex128, 40,000 with mixed precision).  The call allocates nothing (no cudaMalloc, no
 * cudaFree, no allocating library routine, no CUDA graph) and synchronises the stream; it runs
 * with use_graph = 3 whatever prm->use_graph says: cached-connectivity and CSR operators get the
 * persistent kernel, others eager launches.  The first call on a
 * device looks up the array's device address (once per device).  All calls share the array and it keeps the last call's contents (the solver
 * clears what must start at zero): calls that overlap on the GPU (other streams, other threads)
 * race and must not be issued. */
int rq_lobpcg_solve_noalloc(const rq_operator_t *op, const rq_lobpcg_params_t *prm,
                            const void *x0, void *x_out, rq_lobpcg_result_t *res, void *stream);

/* Matvec supplied by the caller: y = A x in value type vtype on `stream`; return 0 on success. */
typedef int (*rq_matvec_fn)(void *ctx, int32_t vtype, const void *x, void *y, void *stream);

/* rq_lobpcg_solve with the matvec supplied by the caller (ground_locg with a callable or a
 * matrix, ground_locg.py:154-157).  Runs without graph capture, one iteration per launch batch. */
int rq_lobpcg_solve_cb(int64_t D, rq_matvec_fn fn, void *ctx, const rq_lobpcg_params_t *prm,
                       void *workspace, const void *x0, void *x_out, rq_lobpcg_result_t *res,
                       void *stream);

/* Lowest eigenpair of a Hermitian 3x3 (row-major complex double [18]) on the device, Cardano as
 * ground_locg.py:438-471: writes lambda to out[0] and the eigenvector (complex) to out[2..7]. */
int rq_eigenpair_3x3(const double *mat, double *out, void *stream);

/* ---- batches of independent problems ------------------------------------------------------ */

#define RQ_BATCH_STATE_BITS 40   /* composite key = (problem << 40) | state; states < 2^40 */

typedef struct rq_batch {
    int32_t  P;                /* number of problems (< 2^24)                                   */
    int32_t  mode;             /* RQ_MODE_FREE or RQ_MODE_CONN                                   */
    const uint64_t *keys;      /* [D] composite keys, strictly increasing (problems in order)   */
    const int64_t  *prow;      /* [P + 1] first row of each problem                              */
    int64_t  D;                /* total rows                                                     */
    void    *hkeys;            /* hash table over the composite keys: 32 << hbits bytes          */
    int32_t *hvals;            /* [4 << hbits]                                                   */
    int32_t  hbits;            /* rq_subspace_sizes(D, 64, &hbits)                               */
    int32_t  pbits;            /* rq_presence_bits(D, 64, &pbits); 0 = no presence bitmap        */
    uint64_t empty_key;        /* written by rq_batch_build                                      */
    const uint64_t *fmask;     /* [2P] sector filter masks (a, b) of each problem; NULL = off    */
    uint32_t *fbits;           /* [P * RQ_FILTER_WORDS], written by rq_batch_build               */
    rq_terms_t terms;          /* every problem's X groups concatenated (toff over all terms)   */
    const int32_t *gofs;       /* [P + 1] first group of each problem                            */
    const int32_t *dgrp;       /* [P] global index of each problem's x = 0 group, or -1          */
    double  *diag0;            /* [D] x = 0 diagonal of each row, written by rq_batch_build      */
    const int64_t *rowptr;     /* [D + 1]  RQ_MODE_CONN                                          */
    const int32_t *col;        /* [nnz]    source row (global index)                             */
    const int32_t *grp;        /* [nnz]    X group (global index)                                */
    int64_t  nnz;
    const int64_t *states_size; /* [P] HOST array: each problem's convergence length (sqd's
                                   states_size, sqd.py:222-225); NULL = its row count        */
    uint32_t *pmap;            /* [2^pbits / 32] presence bitmap over the composite keys       */
    uint32_t *lmap;            /* line filter over the composite keys (as rq_subspace_t.lmap, with
                                  each problem's own prefix shift), or NULL; replaces pmap     */
    uint32_t *xline;           /* [J] written by rq_batch_build: hash(xmask >> shift of the
                                  group's problem)                                           */
    int32_t  *lshift;          /* [P] written by rq_batch_build: each problem's prefix shift    */
    int32_t   lbits;           /* rq_line_filter_bits(D, lwbits, &lbits)                         */
    int32_t   lwbits;          /* 8 .. 10                                                        */
} rq_batch_t;

/* Validate the keys, fill the hash table, the per-problem sector filters and diag0.
 * Synchronises the stream.  Many independent Pauli sums on their own subspaces are solved
 * together: one launch per step serves all problems.  Every X mask must fit in the state bits
 * (below bit RQ_BATCH_STATE_BITS); rq_batch_build rejects one that does not. */
int rq_batch_build(rq_batch_t *b, void *scratch, void *stream);

/* Connectivity of every row (RQ_MODE_CONN), two passes as rq_conn_build. */
int rq_batch_conn_build(const rq_batch_t *b, int64_t *rowptr, int32_t *col, int32_t *grp,
                        int64_t *nnz, void *scratch, void *stream);

/* y = H_p x on every problem's rows at once. */
int rq_batch_matvec(const rq_batch_t *b, int32_t vtype, const void *x, void *y, void *scratch,
                    void *stream);

/* LOBPCG on all problems together (rows of every problem in one vector, per-problem reductions,
 * Rayleigh-Ritz and convergence; converged problems stop).  res has P entries; the convergence
 * test of problem p uses states_size[p] (or its row count). */
int rq_batch_workspace_size(const rq_batch_t *b, const rq_lobpcg_params_t *prm, size_t *bytes);
int rq_batch_solve(const rq_batch_t *b, const rq_lobpcg_params_t *prm, void *workspace,
                   const void *x0, void *x_out, rq_lobpcg_result_t *res, void *stream);

/* ---- learned warm start ------------------------------------------------------------------
 * An MLP f(features) -> (log-amplitude, sign logit) of the ground state, trained on ground
 * states of related problems (the same subspace, another value of a Hamiltonian parameter U)
 * and evaluated on every state of a new problem to give LOBPCG its start vector (replaces the
 * one-hot start of sqd.py:373-398).  Architecture: 64 inputs (the 32 low state bits as +-1,
 * then (U - 5) / 3, its square and cube, zeros), two hidden layers of 256 GELU units, 2
 * outputs.  BF16 weights and activations on the tcgen05 tensor cores (FP32 accumulators in
 * TMEM), FP32 master weights and Adam state.  Row counts of rq_mlp_bwd are multiples of 128. */

#define RQ_MLP_IN 64
#define RQ_MLP_HIDDEN 256
#define RQ_MLP_OUT 2
#define RQ_MLP_NPARAMS (256 * 64 + 256 + 256 * 256 + 256 + 2 * 256 + 2)

typedef struct rq_mlp {
    float    *params;     /* [NPARAMS] FP32: W1[256][64] b1[256] W2[256][256] b2[256] W3[2][256] b3[2] */
    float    *grads;      /* [NPARAMS] written by rq_mlp_bwd (same layout)                      */
    float    *adam_m;     /* [NPARAMS] Adam first moment                                         */
    float    *adam_v;     /* [NPARAMS] Adam second moment                                        */
    uint16_t *w1b;        /* [256][64]  BF16 copy of W1     (rq_mlp_sync / rq_mlp_step)          */
    uint16_t *w2b;        /* [256][256] BF16 copy of W2                                          */
    uint16_t *w2tb;       /* [256][256] BF16 copy of W2 transposed                               */
} rq_mlp_t;

/* Device workspace of rq_mlp_fwd / rq_mlp_bwd for `rows` rows (activations kept for bwd). */
int rq_mlp_workspace_size(int64_t rows, size_t *bytes);
/* Refresh the BF16 weight copies from params. */
int rq_mlp_sync(const rq_mlp_t *m, void *stream);
/* Features of every state for one U: x[D][64] BF16. */
int rq_mlp_features(const uint64_t *states, int64_t D, double U, uint16_t *x, void *stream);
/* Training minibatch: `rows` pairs (problem i, row k) drawn by a counter-based hash of
 * (seed, step, row); features x[rows][64] and xt[64][rows] (BF16), targets tgt[rows][3] =
 * (log(sqrt(D) |psi_i[k]|), sign psi_i[k], weight clamp(D psi_i[k]^2, 0.05, 20)).
 * psi is [P][D] FP32 (each ground state normalised), U is [P]. */
int rq_mlp_sample(const uint64_t *states, int64_t D, const double *U, const float *psi, int32_t P,
                  uint64_t seed, int64_t step, int64_t rows, uint16_t *x, uint16_t *xt, float *tgt,
                  void *stream);
/* out[rows][2] = f(x); keeps the activations in ws for rq_mlp_bwd. */
int rq_mlp_fwd(const rq_mlp_t *m, int64_t rows, const uint16_t *x, float *out, void *ws,
               void *stream);
/* out[rows][2] = f(x) without keeping the activations for rq_mlp_bwd (inference: only the
 * hidden activations that layer 2 reads are written to ws). */
int rq_mlp_infer(const rq_mlp_t *m, int64_t rows, const uint16_t *x, float *out, void *ws,
                 void *stream);
/* dout[rows][2] of the weighted loss mean_i w_i ((o0 - a_i)^2 + softplus(-s_i o1)); the loss
 * itself is written to loss[0] (device double) when loss is not NULL. */
int rq_mlp_loss(int64_t rows, const float *out, const float *tgt, float *dout, double *loss,
                void *ws, void *stream);
/* m->grads = d loss / d params from dout and the activations of the last rq_mlp_fwd on ws. */
int rq_mlp_bwd(const rq_mlp_t *m, int64_t rows, const uint16_t *xt, const float *dout, void *ws,
               void *stream);
/* One training step without the Adam update: forward, loss and backward of a minibatch (rows a
 * multiple of 128; x[rows][64] and xt[64][rows] BF16, tgt[rows][3] as rq_mlp_sample writes them).
 * m->grads = d loss / d params; out[rows][2] = f(x) when out is not NULL; loss[0] (device double)
 * = the loss of rq_mlp_loss when loss is not NULL.  Layer 2's epilogue computes the loss gradient
 * and dZ2 in place (the same gradients as rq_mlp_fwd + rq_mlp_loss + rq_mlp_bwd, with Z2 kept in
 * FP32 rather than rounded to BF16). */
int rq_mlp_train(const rq_mlp_t *m, int64_t rows, const uint16_t *x, const uint16_t *xt,
                 const float *tgt, float *out, double *loss, void *ws, void *stream);
/* One Adam step (step number t >= 1) on params from grads; refreshes the BF16 copies. */
int rq_mlp_step(const rq_mlp_t *m, int32_t t, float lr, float beta1, float beta2, float eps,
                void *stream);
/* Start vector x0[k] = sign(o1_k) exp(o0_k) of value type vtype from out[D][2]. */
int rq_mlp_warm_start(int64_t D, const float *out, int32_t vtype, void *x0, void *stream);
/* The tensor-core GEMM under the MLP: C[M][N] = A[M][K] B[N][K]^T (BF16 in, FP32 out), N 64 or
 * 256, K a multiple of 64, row strides multiples of 8 elements; ws: 16 bytes of device memory
 * (error flag). */
int rq_bf16_gemm(const uint16_t *A, int64_t lda, const uint16_t *B, int64_t ldb, int64_t M,
                 int32_t N, int64_t K, float *C, void *ws, void *stream);

/* ---- state-vector simulation ------------------------------------------------------------- */

/* Apply Pauli-rotation gates in order to a complex128 state of 2^n amplitudes, in place (the
 * reference's svsim, svsim.py:88-122): gate g maps
 *     out[i] = i sin[g] (-1)^popcount(i & z[g]) state[i ^ x[g]] + cos[g] state[i]
 * (the cos term is omitted when cos[g] == 0).  x, z, cos, sin are HOST arrays of ngates
 * entries (the gate list of CircuitXZ, svsim.py:42-49); gates_scratch is device memory of
 * 32 * ngates bytes.  Synchronises the stream. */
int rq_svsim(const uint64_t *x, const uint64_t *z, const double *cos_, const double *sin_,
             int32_t ngates, int32_t n, void *state, void *gates_scratch, void *stream);

/* ---- diagnostics ------------------------------------------------------------------------- */

const char *rq_last_error(void);
int rq_version(void);

#ifdef __cplusplus
}
#endif

#endif /* RQSQD_H */
