/*
 * caps_gb300.h -- C ABI of the GB300 CAPS Strassen multiply library
 * (libcaps_gb300.so).  Plain pointers and sizes only; a stream is passed as
 * `void *` holding a cudaStream_t (NULL = the legacy default stream).
 *
 * Matrices are n x n float64 in CAPS's recursive block layout: `nrec` levels
 * of quadrants stored in the order 11, 21, 12, 22, then bs x bs blocks,
 * column-major both inside a block and between blocks (matrix.h:20-44).
 * With bs = 1 a leaf is a plain column-major (n/2^nrec)^2 matrix.
 *
 * Every entry point returns a caps_status; nothing calls exit().
 */
#ifndef CAPS_GB300_H
#define CAPS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Mirrors struct MatDescriptor (matrix.h:8-16), same field order. */
typedef struct caps_desc {
    int lda;          /* matrix dimension n */
    int nrec;         /* recursive Strassen steps */
    int nproc;        /* must be 1: one GPU holds the whole matrix */
    int nprocr;       /* must be 1 */
    int nprocc;       /* must be 1 */
    int nproc_summa;  /* the reference's P factor (process groups of a hybrid
                         'h' step); on one GPU, the subproducts an 'h' step runs at
                         once: 1 (the step runs as 'd', as the reference does on
                         one rank) or 2..6 (strassenHybrid2..6, multiply.cpp:458-1080:
                         the operands of a 'b' step, its subproducts k at a time) */
    int bs;           /* leaf block size; lda % (2^nrec * bs) == 0 */
} caps_desc;

typedef enum caps_status {
    CAPS_OK = 0,
    CAPS_ERR_INVALID_PATTERN = 1, /* a pattern char other than b/B/d/D/h/H, or too short */
    CAPS_ERR_SIZE = 2,            /* lda not divisible by 2^nrec*bs, or n <= 0 */
    CAPS_ERR_BUDGET = 3,          /* workspace the pattern needs exceeds the -m budget */
    CAPS_ERR_CUDA = 4,            /* a CUDA runtime call failed */
    CAPS_ERR_ALLOC = 5,           /* device memory allocation failed */
    CAPS_ERR_TIMEOUT = 6,         /* a bounded device-side wait gave up */
    CAPS_ERR_UNSUPPORTED = 7,     /* multi-rank descriptor, or no sm_103 device */
    CAPS_ERR_ARG = 8              /* NULL pointer or out-of-range option */
} caps_status;

/* Base-case arithmetic. */
typedef enum caps_form {
    CAPS_FORM_PLAIN = 0, /* FP64 throughout, base case on FP64 DMMA tensor cores */
    CAPS_FORM_SPLIT = 1  /* base case split into int8-valued digit slices with
                            per-row / per-column power-of-two scaling, exact
                            integer slice products on tcgen05, FP64 recombine */
} caps_form;

/* How the split form cuts the base-case operands.  Both scale each row of A
 * and column of B by a power of two into integers of up to 55 bits. */
typedef enum caps_split_scheme {
    CAPS_SPLIT_AUTO = 0,     /* per launch group of leaves: residues wherever the
                                leaves fit them (up to 2048; float and integer
                                data alike, the moduli counted from the data),
                                digits for larger leaves */
    CAPS_SPLIT_DIGITS = 1,   /* balanced base-128 digits, one product per kept
                                digit pair (36 for float data) */
    CAPS_SPLIT_RESIDUES = 2  /* residues modulo up to 17 coprime moduli <= 181,
                                one product per modulus, exact CRT recombination;
                                leaves up to 2048 (larger leaves use digits) */
} caps_split_scheme;

typedef struct caps_options {
    int form;                  /* caps_form */
    int slices;                /* split form: digits per operand, 0 = automatic, 1..8 */
    int diagonals;             /* split form: digit-pair diagonals kept, 0 = automatic */
    int split_scheme;          /* split form: caps_split_scheme */
    long long workspace_limit; /* bytes of device workspace allowed (-m); <= 0: no limit */
    int plain_tile;            /* plain form: the DMMA base case's CTA tile, caps_plain_tile */
    int operand_bits;          /* split form, residue scheme: cap on the operand bits, 0 = 55
                                  (the data's own need when lower); fewer bits take fewer moduli
                                  and round the operands more coarsely.  1..55, or
                                  CAPS_OPERAND_BITS_TUNED */
    long long reserved[3];
} caps_options;

/* caps_options.operand_bits: the library picks 55, 52 or 48 bits per leaf
 * size -- the fewest (fewest moduli: 17 / 16 / 15) that run faster than 55
 * and whose leaf product, on synthetic uniform and wide-range (u 2^k,
 * |k| <= 20) leaves, is no less accurate than the FP64 DMMA leaf's (squared
 * error sum, and largest entry error relative to |A||B|, against a 55-bit
 * reference).  Timed and
 * checked on the device once per leaf size and device, and kept with the
 * autotuner's choices (caps_autotune_info, leaf_gate = 1); make the first
 * such call for a leaf size outside any stream capture. */
#define CAPS_OPERAND_BITS_TUNED (-1)

/* CTA tiles of the plain form's DMMA base case. */
typedef enum caps_plain_tile {
    CAPS_TILE_64x64 = 0,   /* default */
    CAPS_TILE_32x32 = 1,   /* one warp per CTA: four times the CTAs, for small leaves */
    CAPS_TILE_128x64 = 2   /* eight warps: half the B traffic per multiply-add */
} caps_plain_tile;

/* Fills *opt with defaults (plain form, automatic slices, no limit). */
void caps_options_init(caps_options *opt);

/* C = A * B on device-resident CAPS-layout matrices (the `multiply()` of
 * multiply.h:13, multiply.cpp:9-25, with device pointers and a stream).
 * pattern: one char per level ('b'/'B' = the 7 subproducts run concurrently
 * in one launch, 'd'/'D' = in sequence, 'h'/'H' = 'd' on one GPU), or NULL
 * to let the library choose.  Asynchronous on `stream`. */
caps_status caps_multiply_dev(const double *A, const double *B, double *C, caps_desc desc,
                              const char *pattern, const caps_options *opt, void *stream);

/* Same, on host arrays: copies A, B to the device, multiplies, copies C back
 * and synchronises.  Replaces the body of multiply() for host callers. */
caps_status caps_multiply_host(const double *A, const double *B, double *C, caps_desc desc,
                               const char *pattern, const caps_options *opt);

/* Column-major n x n (ld = n) -> CAPS layout, on the device.
 * Replaces distributeFrom1Proc (communication.cpp:612-657) for one rank. */
caps_status caps_to_caps_layout_dev(const double *colmajor, double *caps, caps_desc desc,
                                    void *stream);

/* CAPS layout -> column-major n x n, on the device.
 * Replaces collectTo1Proc (communication.cpp:661-708) for one rank. */
caps_status caps_from_caps_layout_dev(const double *caps, double *colmajor, caps_desc desc,
                                      void *stream);

/* Base case alone: C = A * B for column-major m x m device matrices in the
 * given form (block_multiply -> square_dgemm_zero, multiply.cpp:1082-1141,
 * dgemm-blas.cpp:4-13). */
caps_status caps_leaf_gemm_dev(const double *A, const double *B, double *C, int m,
                               const caps_options *opt, void *stream);

/* Split-form base case C = A * B (column-major m x m, device pointers) that
 * allocates nothing.  No counterpart in the reference.  For callers that
 * cannot let a library call cudaMalloc -- an application whose device memory
 * is all handed to its own pool allocator, or a code path that cannot take
 * the device-wide synchronisation of cudaMalloc / cudaFree.  Its scratch
 * (digit planes, scales, task table, status word) lives in a file-scope
 * device array of 8.5 MiB that every GPU loading the library holds until
 * exit.  Limits: 1 <= m <= 512, otherwise CAPS_ERR_SIZE and nothing runs.
 * slices / diagonals as in caps_options (0 = automatic).  All calls share
 * the array, so calls that overlap on the GPU race: serialise them.  The
 * first call on a device looks up the array's address with that device
 * current and keeps it.  Synchronises `stream` before returning (it reads
 * the kernels' status word back). */
caps_status caps_leaf_gemm_split_noalloc_dev(const double *A, const double *B, double *C, int m,
                                             int slices, int diagonals, void *stream);

/* The Cholesky subproject's multiply, C = alpha * C - A * B^T, on one rank
 * (cholesky/mult.h:6, `mult(C, A, B, n, x, r, alpha)`, mult.cpp:11-28 with
 * x = 1: multBase :76-107 below 1024 or at r = 0, multDFS :109-137 above).
 * n x n matrices in that subproject's recursive layout (cholesky/pack.cpp:
 * 2-49: r levels of quadrants 11, 21, 12, 22, then column-major blocks of
 * n / 2^r) -- the CAPS layout with nrec = r and bs = 1.  The product runs as
 * this library's Strassen-Winograd multiply with r levels (pattern and opt
 * as for caps_multiply_dev); the reference's is classical, so float results
 * differ within the Strassen error bound, and integer-valued data give the
 * same bits.  alpha = 0 leaves C unread (dgemm's beta = 0).  x must be 1
 * (CAPS_ERR_UNSUPPORTED otherwise); n % 2^r != 0 gives CAPS_ERR_SIZE.  C must
 * not overlap A or B.  Device pointers, asynchronous on `stream` apart from
 * the split form's status read. */
caps_status caps_chol_mult_dev(double *C, const double *A, const double *B, int n, int x, int r,
                               double alpha, const char *pattern, const caps_options *opt, void *stream);

/* Same on host arrays: copies in, updates, copies C back, synchronises. */
caps_status caps_chol_mult_host(double *C, const double *A, const double *B, int n, int x, int r,
                                double alpha, const char *pattern, const caps_options *opt);

/* Workspace bytes caps_multiply_dev needs for (desc, pattern, opt). */
caps_status caps_workspace_size(caps_desc desc, const char *pattern, const caps_options *opt,
                                long long *bytes);

/* The pattern the library would run for (desc, pattern, opt): one char per
 * level written to out (at least desc.nrec + 1 bytes). */
caps_status caps_resolve_pattern(caps_desc desc, const char *pattern, const caps_options *opt,
                                 char *out, int out_len);

/* Counters of the last multiply on this thread, as counters.cpp counts them:
 * additions (element ops, incl. base-case m^3), multiplications (m^3 per
 * leaf), and device times in seconds of the add / multiply / reorder phases
 * (CUDA events; 0 unless caps_set_phase_timing(1)). */
typedef struct caps_counters {
    long long additions;
    long long multiplications;
    double time_add;
    double time_mul;
    double time_rearrange;
    long long workspace_peak_bytes;
    int split_slices;        /* digits used by the last split multiply (0 = plain) */
    int split_diagonals;
    long long kernel_launches;
    double time_leaf_gemm;   /* seconds in base-case GEMM kernels alone (phase timing on) */
    long long leaf_gemm_launches;
    double leaf_gemm_m3;     /* sum of leaves * m^3 over those launches */
    long long add_bytes;     /* algorithmic bytes read + written by the sum / combination kernels */
    int split_moduli;        /* moduli used by the last split multiply's residue scheme (0: digits ran) */
    int split_pad;
    /* caps_multiply_host with phase timing on: seconds from the call's start
     * on the device to the first inputs the plan waits for being on the
     * device (A11 and B11, or their first sub-quadrants with two or more
     * levels), to all inputs being on the device, to the last kernel, and to
     * the last C quadrant being back on the host (0 otherwise) */
    double host_first_inputs;
    double host_all_inputs;
    double host_compute_end;
    double host_copy_back_end;
} caps_counters;

void caps_get_counters(caps_counters *out);
void caps_reset_counters(void);
void caps_set_phase_timing(int enable);

/* Batched independent multiplies of uneven sizes.  Matrices i use A[i],
 * B[i], C[i] (device, column-major n[i] x n[i]).  Instances are grouped by
 * size; the autotuner picks depth, b/d pattern, split scheme, DMMA tile and
 * residue operand bits per size (caps_autotune_info; timed on first use,
 * kept per process and on disk), overriding those fields of `opt`; each
 * size class runs as one batched
 * recursion whose base case is a persistent GEMM launch; the whole batch is
 * captured once as a CUDA graph and replayed while the same sizes and
 * pointers come back.  Synchronises `stream` before returning.  No
 * reference counterpart (the reference runs one multiply per process). */
caps_status caps_multiply_batched_dev(int count, const double *const *A, const double *const *B,
                                      double *const *C, const int *n, const caps_options *opt,
                                      void *stream);

/* The rectangular subproject's rectMM on one rank (rect-class/rectmm.h:1,
 * rectmm.cpp:24-72): C = A B by classical recursive blocking, A m x k, B k x n,
 * C m x n in its block layout (at each of the r levels a column-major grid of
 * blocks, divm x divk for A, divk x divn for B, divm x divn for C, by the
 * level's div_pattern triple; base blocks column-major), base case on FP64
 * DMMA.  pattern: r chars, 'd'/'D' (DFS); 'b'/'B' (BFS) needs more than one
 * rank: CAPS_ERR_UNSUPPORTED.  Every division must be exact (CAPS_ERR_SIZE).
 * The result is the reference's on one rank, including its DFS walk: each
 * base case writes its C block with beta = 0, so every k block overwrites
 * the one before, and with divm, divn > 1 blocks of neighbouring columns
 * coincide (the last product wins); blocks the walk never writes keep C's
 * entries.  Device pointers, asynchronous on `stream`. */
caps_status caps_rect_mm_dev(const double *A, const double *B, double *C, int m, int n, int k, int r,
                             const char *pattern, const int *div_pattern, void *stream);

/* The same on host arrays: copies A, B and C in, C back; synchronises. */
caps_status caps_rect_mm_host(const double *A, const double *B, double *C, int m, int n, int k, int r,
                              const char *pattern, const int *div_pattern);

/* Autotuner choices made so far: entry `index` (0, 1, ...) gives the size,
 * form, recursion depth, pattern (8 bytes) and seconds per instance of the
 * winning candidate; CAPS_ERR_ARG past the last entry.  No reference
 * counterpart. */
caps_status caps_autotune_entry(int index, int *n, int *form, int *nrec, char *pattern, double *seconds);

/* The same with the split scheme the tuner chose (caps_split_scheme; 0 for
 * the plain form) and whether the entry was read from the on-disk cache (1)
 * or timed in this process (0).  The tuner searches recursion depth (0..3,
 * as the leaves allow), the top step's b/d pattern and, for the split form
 * with an automatic scheme, residues against digits.  Its choices are kept
 * in CAPS_AUTOTUNE_CACHE (a file; empty: no cache) or by default in
 * $HOME/.cache/caps_gb300/autotune.tsv, keyed by the device's name and SM
 * count, the size, form, slices and asked-for scheme.  Any pointer may be
 * NULL.  caps_autotune_info gives every axis. */
caps_status caps_autotune_entry_ex(int index, int *n, int *form, int *nrec, char *pattern, int *scheme,
                                   int *from_cache, double *seconds);

/* One autotuner choice with all its axes. */
typedef struct {
    int n;              /* matrix size */
    int form;           /* caps_form */
    int nrec;           /* Strassen levels */
    char pattern[8];    /* b/d per level, NUL-terminated */
    int scheme;         /* split form: the scheme chosen (caps_split_scheme); plain form: 0 */
    int tile_rows;      /* CTA tile of the base-case GEMM: plain form 64 x 64, 32 x 32 or */
    int tile_cols;      /*   128 x 64 (searched); residues 128 x 256, digits 128 x 64 (fixed) */
    int operand_bits;   /* residues: operand bits per entry (55, or a smaller cap that won); else 0 */
    int moduli;         /* residues: moduli per leaf product for float data at that cap; else 0 */
    int gate_rejected;  /* residues: smaller bit caps that ran faster but failed the accuracy gate */
    int leaf_gate;      /* 1: the operand-bit choice for single multiplies' leaves of n
                           (CAPS_OPERAND_BITS_TUNED), not a batched size class */
    int from_cache;     /* 1: read from the on-disk cache */
    double seconds;     /* per instance, of the choice */
} caps_tune_info;

/* Autotuner choice `index` (0, 1, ...) with all its axes; CAPS_ERR_ARG past
 * the last entry or for a NULL `out`.  The tuner searches, in turn:
 *   1. recursion depth (0..3 as the leaves allow) and the top step's b/d
 *      pattern, and for the split form with an automatic scheme, residues
 *      against digits;
 *   2. plain form: the DMMA tile;
 *   3. split form where the residues won: operand bits 55 / 52 / 48 (17 / 16 /
 *      15 moduli at K <= 2048), a smaller cap kept only if it is faster and
 *      its error against a split reference is no larger than the plain FP64
 *      form's at the same depth and pattern (normwise, and largest entry
 *      relative to |A||B|), on
 *      uniform and on wide-range (u 2^k, |k| <= 20) synthetic inputs.
 * No reference counterpart. */
caps_status caps_autotune_info(int index, caps_tune_info *out);

/* Human-readable text of a status. */
const char *caps_status_string(caps_status s);

/* Text of the most recent CUDA error seen by this thread ("" if none). */
const char *caps_last_cuda_error(void);

/* Test hook: make the next `count` device allocations fail (host-side fault
 * injection, no GPU fault).  count <= 0 disables. */
void caps_debug_fail_allocations(int count);

/* Test hook for the bounded device waits: the next `count` split-form GEMM
 * launches issue no copies, so their waits have nothing in flight and give up
 * after a short spin; the call returns CAPS_ERR_TIMEOUT, with TMEM freed and
 * the context usable, and the next call runs normally.  No fault, trap or
 * hang is involved.  count <= 0 disables. */
void caps_debug_starve_split_gemm(int count);

/* Test hook for the autotuner's on-disk cache (host only, no device call):
 * 1 if `line`, one line of the cache file, holds a usable choice for size n
 * under (form, slices, split_scheme) on the device whose key is
 * `device_key` (the device name with blanks as '_', '/', its SM count), and
 * then fills *out (if not NULL) as caps_autotune_info would; 0 for a line
 * of another version, device or size, or a damaged one (a field missing or
 * out of range, a pattern that is not nrec steps of 'b' / 'd'). */
int caps_debug_tune_cache_line(const char *line, const char *device_key, int n, int form, int slices,
                               int split_scheme, caps_tune_info *out);

/* Releases cached workspace and plans. */
void caps_release_cache(void);

#ifdef __cplusplus
}
#endif

#endif /* CAPS_GB300_H */
