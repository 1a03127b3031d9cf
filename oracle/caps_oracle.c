/*
 * caps_oracle.c -- CPU oracle for the CAPS Strassen multiply path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA path is
 * compared against (tests, smoke check) and the timed CPU restatement of the
 * reference's own CPU path (the "port" baseline in bench.py).  Nothing in the
 * product library links, loads or calls it.
 *
 * Parity pins: the integer known-answer fixtures of the reference
 * (tests/test{28,42,56,196,294,392}.{in,correct}) and, in the build container,
 * bit-for-bit agreement with the reference's own multiply() compiled unmodified
 * (oracle/build_ref.sh) on random float inputs with the same BLAS.
 *
 * What it restates (file:line in the CAPS sources):
 *   - recursive block layout and its reorder:   communication.cpp:612-704,
 *                                               matrix.h:20-44, matrix.cpp:9-12
 *   - Strassen-Winograd step ('d' and 'b'):     multiply.cpp:409-454 (DFS, OpenMP
 *     variant) and multiply.cpp:212-310 (BFS; per-element identical arithmetic)
 *   - element-wise additions / C combination:   multiply.cpp:110-210
 *   - base case with bs repack:                 multiply.cpp:1082-1141,
 *                                               dgemm-blas.cpp:4-13
 *   - pattern dispatch on one rank:             multiply.cpp:28-108
 *   - the Cholesky subproject's multiply,       cholesky/mult.cpp:11-137,
 *     C = alpha C - A B^T, on one rank:         cholesky/pack.cpp:2-49
 * plus a double-double classical product (Ogita, Rump, Oishi 2005, "Accurate
 * sum and dot product", algorithm Dot2) used as the float oracle, and a CPU
 * model of the split-integer base case that the GPU form must match exactly.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef void (*dgemm_ilp64_fn)(const char *, const char *, const int64_t *,
                               const int64_t *, const int64_t *, const double *,
                               const double *, const int64_t *, const double *,
                               const int64_t *, const double *, double *,
                               const int64_t *);

static dgemm_ilp64_fn g_dgemm = 0;     /* optional BLAS (ILP64 Fortran ABI) */
static int g_threads = 1;

/* Installs an ILP64 Fortran dgemm (e.g. OpenBLAS's scipy_dgemm_64_) as the
 * base-case multiply; NULL restores the built-in classical loop. */
void caps_oracle_set_dgemm(void *fn) { g_dgemm = (dgemm_ilp64_fn)fn; }
void caps_oracle_set_threads(int t) { g_threads = t > 0 ? t : 1; }

/* ---------------------------------------------------------------------- */
/* Layout: index of element (r, c) of an n x n matrix in CAPS block layout  */
/* with nrec recursive levels (quadrant order 11, 21, 12, 22) and bs x bs   */
/* column-major blocks, blocks column-major within the leaf.                */
/* communication.cpp:612-655 (distribute), :661-704 (collect), 1 rank.      */
/* ---------------------------------------------------------------------- */
int64_t caps_oracle_layout_index(int64_t n, int nrec, int64_t bs, int64_t r, int64_t c)
{
    int64_t off = 0, size = n;
    for (int l = 0; l < nrec; l++) {
        int64_t h = size / 2;
        int64_t q = (r >= h ? 1 : 0) + (c >= h ? 2 : 0);
        off += q * h * h;
        if (r >= h) r -= h;
        if (c >= h) c -= h;
        size = h;
    }
    int64_t nb = size / bs;
    off += ((r / bs) + (c / bs) * nb) * bs * bs + (c % bs) * bs + (r % bs);
    return off;
}

/* column-major n x n (ld = n)  ->  CAPS layout.   distributeFrom1Proc. */
void caps_oracle_to_caps(int64_t n, int nrec, int64_t bs, const double *colmajor, double *caps)
{
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int64_t c = 0; c < n; c++)
        for (int64_t r = 0; r < n; r++)
            caps[caps_oracle_layout_index(n, nrec, bs, r, c)] = colmajor[r + c * n];
}

/* CAPS layout -> column-major.   collectTo1Proc. */
void caps_oracle_from_caps(int64_t n, int nrec, int64_t bs, const double *caps, double *colmajor)
{
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int64_t c = 0; c < n; c++)
        for (int64_t r = 0; r < n; r++)
            colmajor[r + c * n] = caps[caps_oracle_layout_index(n, nrec, bs, r, c)];
}

/* ---------------------------------------------------------------------- */
/* Base case: C = A * B for an m x m leaf (multiply.cpp:1082-1141).        */
/* ---------------------------------------------------------------------- */
static void classical_colmajor(int64_t m, const double *A, const double *B, double *C)
{
    /* C(:,j) = sum_k A(:,k) * B(k,j): one rounding per multiply and add,
     * k ascending, like a reference (unblocked) Fortran dgemm. */
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int64_t j = 0; j < m; j++) {
        double *cj = C + j * m;
        for (int64_t i = 0; i < m; i++) cj[i] = 0.0;
        for (int64_t k = 0; k < m; k++) {
            double b = B[k + j * m];
            const double *ak = A + k * m;
            for (int64_t i = 0; i < m; i++) cj[i] += ak[i] * b;
        }
    }
}

static void leaf_dgemm(int64_t m, const double *A, const double *B, double *C)
{
    if (g_dgemm) {
        const char N = 'N';
        const double one = 1.0, zero = 0.0;
        int64_t mm = m;
        g_dgemm(&N, &N, &mm, &mm, &mm, &one, A, &mm, B, &mm, &zero, C, &mm);
    } else {
        classical_colmajor(m, A, B, C);
    }
}

/* block_multiply: repack bs-blocked leaf into column-major when 1<bs<m. */
static void base_case(int64_t m, int64_t bs, const double *A, const double *B, double *C)
{
    if (bs == 1 || bs == m) {
        leaf_dgemm(m, A, B, C);
        return;
    }
    int64_t nb = m / bs, mm = m * m;
    double *w = (double *)malloc((size_t)(3 * mm) * sizeof(double));
    double *AA = w, *BB = w + mm, *CC = w + 2 * mm;
    for (int64_t col = 0; col < m; col++) {
        int64_t cb = col / bs, cr = col % bs;
        for (int64_t rb = 0; rb < nb; rb++) {
            memcpy(AA + col * m + rb * bs, A + (rb + cb * nb) * bs * bs + cr * bs, (size_t)bs * sizeof(double));
            memcpy(BB + col * m + rb * bs, B + (rb + cb * nb) * bs * bs + cr * bs, (size_t)bs * sizeof(double));
        }
    }
    leaf_dgemm(m, AA, BB, CC);
    for (int64_t col = 0; col < m; col++) {
        int64_t cb = col / bs, cr = col % bs;
        for (int64_t rb = 0; rb < nb; rb++)
            memcpy(C + (rb + cb * nb) * bs * bs + cr * bs, CC + col * m + rb * bs, (size_t)bs * sizeof(double));
    }
    free(w);
}

/* ---------------------------------------------------------------------- */
/* One Strassen-Winograd step on CAPS layout, multiply.cpp:409-454.        */
/* Quadrant offsets 0,1,2,3 x q for X11, X21, X12, X22 (multiply.cpp:334). */
/* ---------------------------------------------------------------------- */
static int64_t g_adds = 0, g_muls = 0;

/* Bounded-sample mode for the CPU baseline: at the top level, run every
 * operand sum and C combination but recurse into only subproduct
 * g_sample_child (1..7); the seconds spent in sums and in that one
 * recursion are recorded.  0 = normal operation. */
static int g_sample_child = 0;
static double g_sample_t_top = 0.0, g_sample_t_sub = 0.0;

static double now_s(void)
{
#ifdef _OPENMP
    return omp_get_wtime();
#else
    return 0.0;
#endif
}

static void rec(const double *A, const double *B, double *C, int64_t n, int nrec, int64_t bs,
                const char *pattern);

static void step(const double *A, const double *B, double *C, int64_t n, int nrec, int64_t bs,
                 const char *pattern)
{
    const int sample = g_sample_child;
    g_sample_child = 0; /* only the top level samples */
    double t_enter = now_s(), t_in_rec = 0.0;
#define REC(child, a, b, c)                                                   \
    do {                                                                      \
        if (!sample || sample == (child)) {                                   \
            double _t0 = now_s();                                             \
            rec(a, b, c, h, nrec - 1, bs, pattern);                           \
            if (sample) { g_sample_t_sub = now_s() - _t0; t_in_rec += g_sample_t_sub; } \
        }                                                                     \
    } while (0)
    int64_t h = n / 2, q = h * h;
    const double *A11 = A, *A21 = A + q, *A12 = A + 2 * q, *A22 = A + 3 * q;
    const double *B11 = B, *B21 = B + q, *B12 = B + 2 * q, *B22 = B + 3 * q;
    double *C11 = C, *C21 = C + q, *C12 = C + 2 * q, *C22 = C + 3 * q;
    double *W = (double *)malloc((size_t)(9 * q) * sizeof(double));
    double *T3 = W, *T4 = W + q, *T5 = W + 2 * q, *T6 = W + 3 * q;
    double *S3 = W + 4 * q, *S4 = W + 5 * q, *S5 = W + 6 * q, *S7 = W + 7 * q;
    double *Qt = W + 8 * q;
    /* S/T sums: same per-element formulas and order as the reference
     * (tripleSubMatrices/addSubMatrices/subMatrices, :421-435). */
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int64_t i = 0; i < q; i++) {
        S5[i] = B22[i] - B12[i];
        S3[i] = B12[i] - B11[i];
        S4[i] = B22[i] - S3[i];
        T3[i] = A21[i] + A22[i];
        T5[i] = A11[i] - A21[i];
        T4[i] = T3[i] - A11[i];
        T6[i] = A12[i] - T4[i];
        S7[i] = S4[i] - B21[i];
    }
    g_adds += 8 * q;
    /* Q1 -> C11 (kept as Q1 until C11 = Q1 + Q2). The C combination
     * (calcCij, :195-210 / :444-451):
     *   C11 = Q1+Q2;  U1 = Q1+Q4;  U2 = U1+Q5;  C21 = U2-Q7;  C22 = U2+Q3;
     *   U3 = U1+Q3;   C12 = U3+Q6. */
    double *U = (double *)malloc((size_t)(2 * q) * sizeof(double));
    double *U2 = U, *U3 = U + q;
    REC(1, A11, B11, C11);                                  /* Q1 in C11 */
    REC(4, T4, S4, Qt);                                     /* Q4 */
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int64_t i = 0; i < q; i++) { double u1 = C11[i] + Qt[i]; U2[i] = u1; U3[i] = u1; }
    REC(5, T5, S5, Qt);                                     /* Q5 */
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int64_t i = 0; i < q; i++) U2[i] = U2[i] + Qt[i];
    REC(3, T3, S3, Qt);                                     /* Q3 */
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int64_t i = 0; i < q; i++) { C22[i] = U2[i] + Qt[i]; U3[i] = U3[i] + Qt[i]; }
    REC(7, A22, S7, Qt);                                    /* Q7 */
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int64_t i = 0; i < q; i++) C21[i] = U2[i] - Qt[i];
    REC(6, T6, B22, Qt);                                    /* Q6 */
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int64_t i = 0; i < q; i++) C12[i] = U3[i] + Qt[i];
    REC(2, A12, B21, Qt);                                   /* Q2 */
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int64_t i = 0; i < q; i++) C11[i] = C11[i] + Qt[i];
    g_adds += 7 * q;
    free(U);
    free(W);
    if (sample) g_sample_t_top = (now_s() - t_enter) - t_in_rec;
#undef REC
}

static int g_bad_pattern = 0;

/* multiplyInternal on one rank (multiply.cpp:28-108): 'b','d','h' (and NULL)
 * all perform the same per-element Winograd arithmetic on one process. */
static void rec(const double *A, const double *B, double *C, int64_t n, int nrec, int64_t bs,
                const char *pattern)
{
    if (nrec == 0) {
        g_adds += n * n * n;
        g_muls += n * n * n;
        base_case(n, bs, A, B, C);
        return;
    }
    if (pattern) {
        char p = pattern[0];
        if (!(p == 'b' || p == 'B' || p == 'd' || p == 'D' || p == 'h' || p == 'H')) {
            g_bad_pattern = 1;
            return;
        }
        pattern++;
    }
    step(A, B, C, n, nrec, bs, pattern);
}

/* multiply() on one rank (multiply.cpp:9-25).  Returns 0, or -1 for an
 * invalid pattern character, -2 for a size the layout cannot hold. */
int caps_oracle_multiply(const double *A, const double *B, double *C, int64_t n, int nrec,
                         int64_t bs, const char *pattern)
{
    if (n <= 0 || nrec < 0 || bs <= 0 || (n % (((int64_t)1 << nrec) * bs)) != 0) return -2;
    g_bad_pattern = 0;
    rec(A, B, C, n, nrec, bs, pattern);
    return g_bad_pattern ? -1 : 0;
}

/* Bounded sample of a multiply for the CPU baseline: all top-level sums and
 * combinations, one of the seven subproducts (child 1..7) in full.  Returns
 * the seconds in top-level sums and in the subproduct; the full run takes
 * about t_top + 7 t_sub.  C holds no meaningful result afterwards. */
int caps_oracle_multiply_sample(const double *A, const double *B, double *C, int64_t n, int nrec,
                                int64_t bs, const char *pattern, int child, double *t_top,
                                double *t_sub)
{
    if (nrec < 1 || child < 1 || child > 7) return -2;
    g_sample_child = child;
    g_sample_t_top = g_sample_t_sub = 0.0;
    int rc = caps_oracle_multiply(A, B, C, n, nrec, bs, pattern);
    g_sample_child = 0;
    *t_top = g_sample_t_top;
    *t_sub = g_sample_t_sub;
    return rc;
}

/* add/multiply counters as the reference counts them (counters.cpp). */
void caps_oracle_counters(int64_t *adds, int64_t *muls) { *adds = g_adds; *muls = g_muls; }
void caps_oracle_reset_counters(void) { g_adds = 0; g_muls = 0; }

/* ---------------------------------------------------------------------- */
/* The Cholesky subproject's multiply on one rank: C = alpha C - A B^T.    */
/* cholesky/mult.cpp:11-28 (dispatch, x = 1), multBase :76-107, multDFS    */
/* :109-137, pack / unpack cholesky/pack.cpp:2-49.  Its recursive layout   */
/* is the CAPS layout above with nrec = r, bs = 1.  At r = 0 or n <= 1024  */
/* (the reference's minsize) the block is unpacked to column-major and     */
/* updated by one dgemm('N', 'T', alpha = -1, beta = alpha); above, the    */
/* eight quadrant updates run in the reference's order, the first of each  */
/* pair with alpha and the second with 1.  alpha = 0 leaves C unread.      */
/* ---------------------------------------------------------------------- */
static const int64_t CHOL_MINSIZE = 1024;   /* mult.cpp:9 */

static void chol_base(int64_t n, int r, double alpha, double *C, const double *A, const double *B)
{
    int64_t nn = n * n;
    double *w = r ? (double *)malloc((size_t)(3 * nn) * sizeof(double)) : 0;
    const double *AA = A, *BB = B;
    double *CC = C;
    if (r) {
        double *a = w, *b = w + nn;
        CC = w + 2 * nn;
        caps_oracle_from_caps(n, r, 1, A, a);
        caps_oracle_from_caps(n, r, 1, B, b);
        if (alpha != 0.0) caps_oracle_from_caps(n, r, 1, C, CC);
        AA = a;
        BB = b;
    }
    if (g_dgemm) {
        const char N = 'N', T = 'T';
        const double none = -1.0;
        g_dgemm(&N, &T, &n, &n, &n, &none, AA, &n, BB, &n, &alpha, CC, &n);
    } else {
        /* rows of A and of B made contiguous, k ascending in each sum */
        double *at = (double *)malloc((size_t)(2 * nn) * sizeof(double)), *bt = at + nn;
        for (int64_t k = 0; k < n; k++)
            for (int64_t i = 0; i < n; i++) {
                at[i * n + k] = AA[i + k * n];
                bt[i * n + k] = BB[i + k * n];
            }
#pragma omp parallel for num_threads(g_threads) schedule(static)
        for (int64_t j = 0; j < n; j++)
            for (int64_t i = 0; i < n; i++) {
                double acc = 0.0;
                const double *a = at + i * n, *b = bt + j * n;
                for (int64_t k = 0; k < n; k++) acc += a[k] * b[k];
                double c = alpha == 0.0 ? 0.0 : alpha * CC[i + j * n];
                CC[i + j * n] = c - acc;
            }
        free(at);
    }
    if (r) {
        caps_oracle_to_caps(n, r, 1, CC, C);
        free(w);
    }
}

void caps_oracle_chol_mult(double *C, const double *A, const double *B, int64_t n, int r, double alpha)
{
    if (r == 0 || n <= CHOL_MINSIZE) {
        chol_base(n, r, alpha, C, A, B);
        return;
    }
    int64_t h = n / 2, q = h * h;
    double *C11 = C, *C21 = C + q, *C12 = C + 2 * q, *C22 = C + 3 * q;
    const double *A11 = A, *A21 = A + q, *A12 = A + 2 * q, *A22 = A + 3 * q;
    const double *B11 = B, *B21 = B + q, *B12 = B + 2 * q, *B22 = B + 3 * q;
    caps_oracle_chol_mult(C11, A11, B11, h, r - 1, alpha);
    caps_oracle_chol_mult(C11, A12, B12, h, r - 1, 1.0);
    caps_oracle_chol_mult(C12, A11, B21, h, r - 1, alpha);
    caps_oracle_chol_mult(C12, A12, B22, h, r - 1, 1.0);
    caps_oracle_chol_mult(C21, A21, B11, h, r - 1, alpha);
    caps_oracle_chol_mult(C21, A22, B12, h, r - 1, 1.0);
    caps_oracle_chol_mult(C22, A21, B21, h, r - 1, alpha);
    caps_oracle_chol_mult(C22, A22, B22, h, r - 1, 1.0);
}

/* ---------------------------------------------------------------------- */
/* Double-double classical product (Dot2 of Ogita-Rump-Oishi):             */
/* result as if accumulated in twice the working precision.  Column-major. */
/* ---------------------------------------------------------------------- */
static inline void two_sum(double a, double b, double *s, double *e)
{
    double x = a + b, z = x - a;
    *s = x;
    *e = (a - (x - z)) + (b - z);
}

static inline void dot2_acc(double a, double b, double *s, double *c)
{
    double p = a * b;
    double pe = fma(a, b, -p);
    double t, te;
    two_sum(*s, p, &t, &te);
    *s = t;
    *c += te + pe;
}

/* hi/lo of sum_k A(i,k) B(k,j) for every (i, j); A, B column-major n x n. */
void caps_oracle_dd_gemm(int64_t n, const double *A, const double *B, double *Chi, double *Clo)
{
    double *At = (double *)malloc((size_t)(n * n) * sizeof(double));
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int64_t i = 0; i < n; i++)
        for (int64_t k = 0; k < n; k++) At[k + i * n] = A[i + k * n];
#pragma omp parallel for num_threads(g_threads) schedule(dynamic, 4)
    for (int64_t j = 0; j < n; j++) {
        const double *bj = B + j * n;
        for (int64_t i = 0; i < n; i++) {
            const double *ai = At + i * n;
            double s = 0.0, c = 0.0;
            for (int64_t k = 0; k < n; k++) dot2_acc(ai[k], bj[k], &s, &c);
            double hi = s + c;
            Chi[i + j * n] = hi;
            Clo[i + j * n] = c - (hi - s);
        }
    }
    free(At);
}

/* Sampled entries of the same product: rows[t], cols[t] for t < count. */
void caps_oracle_dd_entries(int64_t n, const double *A, const double *B, const int64_t *rows,
                            const int64_t *cols, int64_t count, double *hi, double *lo)
{
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int64_t t = 0; t < count; t++) {
        int64_t i = rows[t], j = cols[t];
        double s = 0.0, c = 0.0;
        for (int64_t k = 0; k < n; k++) dot2_acc(A[i + k * n], B[k + j * n], &s, &c);
        double h = s + c;
        hi[t] = h;
        lo[t] = c - (h - s);
    }
}

/* |A||B| entries (classical, double), used to normalise element-wise error. */
void caps_oracle_absprod_entries(int64_t n, const double *A, const double *B, const int64_t *rows,
                                 const int64_t *cols, int64_t count, double *out)
{
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int64_t t = 0; t < count; t++) {
        int64_t i = rows[t], j = cols[t];
        double s = 0.0;
        for (int64_t k = 0; k < n; k++) s += fabs(A[i + k * n]) * fabs(B[k + j * n]);
        out[t] = s;
    }
}

/* ---------------------------------------------------------------------- */
/* CPU model of the split-integer base case (the GPU "split" form).        */
/* Not a reference algorithm: the reference has only the FP64 dgemm.  It   */
/* states the exact integer arithmetic the GPU kernel performs, so the two */
/* must agree bit for bit.                                                 */
/*                                                                         */
/* Row i of A is scaled by 2^fa[i], column j of B by 2^fb[j], with         */
/* fa = 55 - Ea (|a| < 2^Ea over the row), rounded to integers X (|X| <=    */
/* 2^55) and cut into s balanced base-128 digits d_1..d_s (|d| <= 64),     */
/* most significant first.  The product keeps the digit pairs (a, b) with  */
/* a + b <= nd + 1; pair sums are exact integers.  Diagonals t = a + b are */
/* combined as hi = sum_{t<=5} c_t 2^(7(5-t)), lo = sum_{t>=6} c_t         */
/* 2^(7(9-t)), and the leaf value is (hi 2^28 + lo) 2^(7(s_ref)) 2^-(fa+fb) */
/* rounded once.                                                           */
/* ---------------------------------------------------------------------- */
#define SPLIT_BETA 7

/* exponent E with |x| < 2^E, read from the IEEE exponent field (subnormals
 * count as 2^-1022); -100000 for zero.  Same rule as the GPU slicer. */
static int exp_bound(double x)
{
    uint64_t u;
    memcpy(&u, &x, 8);
    int field = (int)((u >> 52) & 0x7ff);
    if ((u & 0x7fffffffffffffffULL) == 0) return -100000;
    if (field == 0) return -1022;
    return field - 1022;
}

/* digits of round(x * 2^f) in balanced base 128, s digits, MS first. */
static void split_digits(double x, int f, int s, int *d)
{
    /* X = round-half-even(x 2^f) as int64; |X| <= 2^55 by construction */
    double y = ldexp(x, f);
    int64_t X = (int64_t)nearbyint(y);
    /* least significant digit first */
    int64_t R = X;
    int tmp[16];
    int total = 8; /* 8 digits cover 56 bits */
    for (int k = 0; k < total; k++) {
        int64_t low = R & 127;         /* 0..127 (two's complement ok) */
        if (low >= 64) low -= 128;     /* balanced: -64..63 */
        tmp[k] = (int)low;
        R = (R - low) >> 7;            /* exact */
    }
    /* a top carry can leave R = +-1 only when |X| > 2^55 - 2^48*64; we
     * keep |X| <= 2^55 so fold it into the top digit (then |d_1| <= 64). */
    tmp[total - 1] += (int)(R * 128);
    for (int k = 0; k < s; k++) d[k] = tmp[total - 1 - k];
}

/* C_leaf = split product of column-major m x m A and B (nd diagonals kept). */
void caps_oracle_split_gemm(int64_t m, const double *A, const double *B, int s, int nd, double *C)
{
    int *fa = (int *)malloc((size_t)m * sizeof(int));
    int *fb = (int *)malloc((size_t)m * sizeof(int));
    for (int64_t i = 0; i < m; i++) {
        int E = -100000;
        for (int64_t k = 0; k < m; k++) { int e = exp_bound(A[i + k * m]); if (e > E) E = e; }
        fa[i] = (E == -100000) ? 0 : 55 - E;
    }
    for (int64_t j = 0; j < m; j++) {
        int E = -100000;
        for (int64_t k = 0; k < m; k++) { int e = exp_bound(B[k + j * m]); if (e > E) E = e; }
        fb[j] = (E == -100000) ? 0 : 55 - E;
    }
    int8_t *da = (int8_t *)malloc((size_t)(m * m * s));
    int8_t *db = (int8_t *)malloc((size_t)(m * m * s));
    for (int64_t i = 0; i < m; i++)
        for (int64_t k = 0; k < m; k++) {
            int d[16];
            split_digits(A[i + k * m], fa[i], s, d);
            for (int a = 0; a < s; a++) da[(i * m + k) * s + a] = (int8_t)d[a];
        }
    for (int64_t j = 0; j < m; j++)
        for (int64_t k = 0; k < m; k++) {
            int d[16];
            split_digits(B[k + j * m], fb[j], s, d);
            for (int b = 0; b < s; b++) db[(j * m + k) * s + b] = (int8_t)d[b];
        }
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int64_t j = 0; j < m; j++) {
        for (int64_t i = 0; i < m; i++) {
            int64_t ct[20];
            for (int t = 0; t < 20; t++) ct[t] = 0;
            for (int64_t k = 0; k < m; k++) {
                const int8_t *pa = da + (i * m + k) * s, *pb = db + (j * m + k) * s;
                for (int a = 0; a < s; a++)
                    for (int b = 0; b < s; b++)
                        if (a + b + 2 <= nd + 1) ct[a + b + 2] += (int64_t)pa[a] * pb[b];
            }
            int64_t hi = 0, lo = 0;
            for (int t = 2; t <= 5; t++) hi += ct[t] << (7 * (5 - t));
            for (int t = 6; t <= 9; t++) lo += ct[t] << (7 * (9 - t));
            /* value = (hi 2^28 + lo) 2^(7*7) 2^-(fa+fb); one rounding */
            double v = fma((double)hi, 268435456.0, (double)lo);
            C[i + j * m] = ldexp(v, 49 - fa[i] - fb[j]);
        }
    }
    free(da); free(db); free(fa); free(fb);
}

/* ---------------------------------------------------------------------- */
/* CPU model of the residue scheme of the split base case.                 */
/* Not a reference algorithm either.  The GPU computes the product of the  */
/* scaled integers exactly through residues modulo small coprime moduli;   */
/* the model computes the same integer product directly in 128-bit         */
/* integers, independent of the moduli, and rounds it the same way.        */
/*                                                                         */
/* Per row i of A: E_i = max exponent bound, lsb_i = min lowest set bit;   */
/* t_a = min(max_i (E_i - lsb_i + 1), 55), fa_i = t_a - E_i, and           */
/* X_ik = round-half-even(a_ik 2^fa_i); the same per column of B.          */
/* C_ij = sum_k X_ik Y_kj (exact) times 2^-(fa_i + fb_j), rounded once to   */
/* the nearest double (ties to even, subnormals included).                 */
/* ---------------------------------------------------------------------- */

/* exponent of the lowest set bit of x != 0 */
static int low_bit(double x)
{
    uint64_t u;
    memcpy(&u, &x, 8);
    int field = (int)((u >> 52) & 0x7ff);
    uint64_t mant = u & 0xFFFFFFFFFFFFFULL;
    if (field == 0) return -1074 + __builtin_ctzll(mant);
    return field - 1075 + __builtin_ctzll(mant | (1ULL << 52));
}

/* |v| 2^e rounded to the nearest double (ties to even), signed */
static double round_scaled_i128(__int128 v, int e)
{
    if (v == 0) return 0.0;
    int neg = v < 0;
    unsigned __int128 mag = neg ? (unsigned __int128)(-v) : (unsigned __int128)v;
    int nb = 0;
    while (nb < 128 && (mag >> nb) != 0) nb++;
    int sh = nb - 53;
    if (nb - 1 + e < -1022) sh = -1074 - e;
    uint64_t mant;
    int ex;
    if (sh <= 0) {
        mant = (uint64_t)mag;
        ex = e;
    } else if (sh >= 128) {
        mant = 0;
        ex = e;
    } else {
        unsigned __int128 q = mag >> sh, rem = mag - (q << sh), half = (unsigned __int128)1 << (sh - 1);
        mant = (uint64_t)q;
        if (rem > half || (rem == half && (mant & 1))) mant++;
        ex = e + sh;
    }
    double r = ldexp((double)mant, ex);
    return neg ? -r : r;
}

/* scale exponents of the rows of a column-major m x m matrix taken as rows
 * (side 0: rows of A, element (i,k) at i + k m) or as columns (side 1:
 * columns of B, element (k,j) at k + j m); returns max bits over the lines */
static int residue_scales(int64_t m, const double *X, int side, int *E)
{
    int bits = 0;
    for (int64_t r = 0; r < m; r++) {
        int e = -100000, lb = 100000;
        for (int64_t k = 0; k < m; k++) {
            double x = side == 0 ? X[r + k * m] : X[k + r * m];
            if (x == 0.0) continue;
            int eb = exp_bound(x), l = low_bit(x);
            if (eb > e) e = eb;
            if (l < lb) lb = l;
        }
        E[r] = e;
        if (e != -100000 && e - lb + 1 > bits) bits = e - lb + 1;
    }
    return bits;
}

/* The same with the operand bits capped at `cap` (1..55) instead of 55:
 * t_a = min(bits the rows need, cap), likewise t_b. */
void caps_oracle_split_gemm_residues_bits(int64_t m, const double *A, const double *B, double *C, int *t_out,
                                          int cap)
{
    int *Ea = (int *)malloc((size_t)m * sizeof(int));
    int *Eb = (int *)malloc((size_t)m * sizeof(int));
    int ta = residue_scales(m, A, 0, Ea), tb = residue_scales(m, B, 1, Eb);
    if (cap < 1 || cap > 55) cap = 55;
    if (ta > cap) ta = cap;
    if (tb > cap) tb = cap;
    if (t_out) { t_out[0] = ta; t_out[1] = tb; }
    int64_t *X = (int64_t *)malloc((size_t)(m * m) * sizeof(int64_t));  /* row-major X[i][k] */
    int64_t *Y = (int64_t *)malloc((size_t)(m * m) * sizeof(int64_t));  /* Y[j][k] */
    for (int64_t i = 0; i < m; i++)
        for (int64_t k = 0; k < m; k++)
            X[i * m + k] = Ea[i] == -100000 ? 0 : (int64_t)nearbyint(ldexp(A[i + k * m], ta - Ea[i]));
    for (int64_t j = 0; j < m; j++)
        for (int64_t k = 0; k < m; k++)
            Y[j * m + k] = Eb[j] == -100000 ? 0 : (int64_t)nearbyint(ldexp(B[k + j * m], tb - Eb[j]));
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int64_t j = 0; j < m; j++) {
        for (int64_t i = 0; i < m; i++) {
            __int128 acc = 0;
            const int64_t *x = X + i * m, *y = Y + j * m;
            for (int64_t k = 0; k < m; k++) acc += (__int128)x[k] * y[k];
            double v = 0.0;
            if (Ea[i] != -100000 && Eb[j] != -100000)
                v = round_scaled_i128(acc, -((ta - Ea[i]) + (tb - Eb[j])));
            C[i + j * m] = v;
        }
    }
    free(X); free(Y); free(Ea); free(Eb);
}

void caps_oracle_split_gemm_residues(int64_t m, const double *A, const double *B, double *C, int *t_out)
{
    caps_oracle_split_gemm_residues_bits(m, A, B, C, t_out, 55);
}

/* ---------------------------------------------------------------------- */
/* The rectangular subproject's rectMM on one rank (rect-class/rectmm.cpp). */
/* Not Strassen: a classical recursive blocking.  Layout (rectmm.cpp:6-19   */
/* with P = 1): at each level the m x k matrix A is a column-major grid of  */
/* divm x divk blocks (block (M, K) at (M + K divm) x its size), B a grid  */
/* of divk x divn, C of divm x divn; the base blocks are column-major.      */
/* dispatch recRectMM :29-45 (r = 0: the base case; 'b'/'B' a BFS step,     */
/* which one rank cannot take: the caller rejects it; 'd'/'D' a DFS step);  */
/* base case localRectMM :47-51, dgemm with beta = 0; DFS step rectDFS      */
/* :53-72, restated with its pointer walk: A advances one block per (M, K), */
/* B one block per (K, N), C restarts at each K and advances one block per  */
/* M, and one block (not divm blocks) per N.  So on one rank each K block   */
/* overwrites the C block of the one before, and with divm > 1 and divn > 1 */
/* the C blocks of neighbouring columns overlap: the last write wins.       */
/* ---------------------------------------------------------------------- */
static void rect_base(int64_t m, int64_t n, int64_t k, const double *A, const double *B, double *C)
{
    if (g_dgemm) {
        const char N = 'N';
        const double one = 1.0, zero = 0.0;
        g_dgemm(&N, &N, &m, &n, &k, &one, A, &m, B, &k, &zero, C, &m);
        return;
    }
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int64_t j = 0; j < n; j++) {
        double *cj = C + j * m;
        for (int64_t i = 0; i < m; i++) cj[i] = 0.0;
        for (int64_t kk = 0; kk < k; kk++) {
            const double b = B[kk + j * k];
            const double *ak = A + kk * m;
            for (int64_t i = 0; i < m; i++) cj[i] += ak[i] * b;
        }
    }
}

static void rect_rec(const double *A, const double *B, double *C, int64_t m, int64_t n, int64_t k, int r,
                     const char *patt, const int *div)
{
    if (r == 0) {
        rect_base(m, n, k, A, B, C);
        return;
    }
    const int divm = div[0], divn = div[1], divk = div[2];
    const int64_t newm = m / divm, newn = n / divn, newk = k / divk;
    const int64_t subA = newm * newk, subB = newn * newk, subC = newm * newn;
    for (int N = 0; N < divn; N++) {
        const double *Ap = A;
        for (int K = 0; K < divk; K++) {
            double *Cp = C;
            for (int M = 0; M < divm; M++) {
                rect_rec(Ap, B, Cp, newm, newn, newk, r - 1, patt + 1, div + 3);
                Ap += subA;
                Cp += subC;
            }
            B += subB;
        }
        C += subC;
    }
}

/* C = the one-rank rectMM of A (m x k) and B (k x n), patt 'd'/'D' only,
 * every division exact.  Returns 0, or -1 for a pattern it cannot run. */
int caps_oracle_rect_mm(const double *A, const double *B, double *C, int64_t m, int64_t n, int64_t k, int r,
                        const char *patt, const int *div)
{
    for (int l = 0; l < r; l++)
        if (patt[l] != 'd' && patt[l] != 'D') return -1;
    rect_rec(A, B, C, m, n, k, r, patt, div);
    return 0;
}
