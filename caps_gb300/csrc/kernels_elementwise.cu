// Elementwise kernels of the Strassen-Winograd step and the layout reorder.
//
// Operand sums and the C combination follow the reference's per-element
// formulas and evaluation order exactly (multiply.cpp:409-454 for the 'd'
// step, calcCij multiply.cpp:195-210 for the 'b' step), so for identical
// subproducts the GPU result is bit-identical to the reference's.
//
// All of these are HBM-bound streams: 8 bytes per element per operand.  A
// block handles one task (blockIdx.y) and a grid-stride range of elements;
// when every pointer of the launch is 16-byte aligned and q is even, the
// loop moves double2 vectors.
#include "common.cuh"

namespace caps {

// Winograd operand sums (reference order, multiply.cpp:421-435):
//   S5 = B22-B12; S3 = B12-B11; S4 = B22-S3; T3 = A21+A22; T5 = A11-A21;
//   T4 = T3-A11;  T6 = A12-T4;  S7 = S4-B21.
// src: A11 A21 A12 A22 B11 B21 B12 B22 ; dst: T3 T4 T5 T6 S3 S4 S5 S7
__device__ __forceinline__ void form_st(double a11, double a21, double a12, double a22,
                                        double b11, double b21, double b12, double b22,
                                        double *o) {
    double s5 = b22 - b12;
    double s3 = b12 - b11;
    double s4 = b22 - s3;
    double t3 = a21 + a22;
    double t5 = a11 - a21;
    double t4 = t3 - a11;
    double t6 = a12 - t4;
    double s7 = s4 - b21;
    o[0] = t3; o[1] = t4; o[2] = t5; o[3] = t6;
    o[4] = s3; o[5] = s4; o[6] = s5; o[7] = s7;
}

// calcCij (multiply.cpp:195-210).  src Q1..Q7 ; dst C11 C12 C21 C22
__device__ __forceinline__ void calc_cij(const double *q, double *c) {
    double c11 = q[0] + q[1];
    double u1 = q[0] + q[3];
    double u2 = u1 + q[4];
    double c21 = u2 - q[6];
    double c22 = u2 + q[2];
    double u3 = u1 + q[2];
    double c12 = u3 + q[5];
    c[0] = c11; c[1] = c12; c[2] = c21; c[3] = c22;
}

// Operand sums of the memory-lean 'd' step: the same formulas, in the same
// evaluation order, as the reference's (multiply.cpp:421-435).
template <int OP>
__device__ __forceinline__ void form_lean(double a11, double a21, double a12, double a22, double b11,
                                          double b21, double b12, double b22, double &o0, double &o1) {
    if (OP == EW_FORM_T4S4) {
        double t3 = a21 + a22;
        o0 = t3 - a11;
        double s3 = b12 - b11;
        o1 = b22 - s3;
    } else if (OP == EW_FORM_T5S5) {
        o0 = a11 - a21;
        o1 = b22 - b12;
    } else if (OP == EW_FORM_T3S3) {
        o0 = a21 + a22;
        o1 = b12 - b11;
    } else if (OP == EW_FORM_S7) {
        double s3 = b12 - b11;
        double s4 = b22 - s3;
        o0 = s4 - b21;
        o1 = 0.0;
    } else {  // EW_FORM_T6
        double t3 = a21 + a22;
        double t4 = t3 - a11;
        o0 = a12 - t4;
        o1 = 0.0;
    }
}

// which of A11 A21 A12 A22 B11 B21 B12 B22 a lean formula reads
template <int OP>
__host__ __device__ constexpr bool lean_reads(int k) {
    return OP == EW_FORM_T4S4   ? (k == 0 || k == 1 || k == 3 || k == 4 || k == 6 || k == 7)
           : OP == EW_FORM_T5S5 ? (k == 0 || k == 1 || k == 6 || k == 7)
           : OP == EW_FORM_T3S3 ? (k == 1 || k == 3 || k == 4 || k == 6)
           : OP == EW_FORM_S7   ? (k == 4 || k == 5 || k == 6 || k == 7)
                                : (k == 0 || k == 1 || k == 2 || k == 3);
}

template <int OP>
__device__ __forceinline__ void ew_scalar(const EwTask &t, int64_t i) {
    if (OP == EW_FORM_ST) {
        double o[8];
        form_st(t.src[0][i], t.src[1][i], t.src[2][i], t.src[3][i], t.src[4][i], t.src[5][i],
                t.src[6][i], t.src[7][i], o);
#pragma unroll
        for (int k = 0; k < 8; k++) t.dst[k][i] = o[k];
    } else if (OP == EW_COPY) {
        t.dst[0][i] = t.src[0][i];
    } else if (OP == EW_ADD_DUP) {
        double v = t.src[0][i] + t.src[1][i];
        t.dst[0][i] = v;
        t.dst[1][i] = v;
    } else if (OP == EW_ADD) {
        t.dst[0][i] = t.src[0][i] + t.src[1][i];
    } else if (OP == EW_SUB) {
        t.dst[0][i] = t.src[0][i] - t.src[1][i];
    } else if (OP == EW_ADD2) {
        double q = t.src[2][i];
        double a = t.src[0][i] + q;
        double b = t.src[1][i] + q;
        t.dst[0][i] = a;
        t.dst[1][i] = b;
    } else if (OP == EW_CALC_CIJ) {
        double q[7], c[4];
#pragma unroll
        for (int k = 0; k < 7; k++) q[k] = t.src[k][i];
        calc_cij(q, c);
#pragma unroll
        for (int k = 0; k < 4; k++) t.dst[k][i] = c[k];
    } else if (OP >= EW_FORM_T4S4 && OP <= EW_FORM_T6) {
        double v[8], o0, o1;
#pragma unroll
        for (int k = 0; k < 8; k++) v[k] = lean_reads<OP>(k) ? t.src[k][i] : 0.0;
        form_lean<OP>(v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], o0, o1);
        t.dst[0][i] = o0;
        if (OP <= EW_FORM_T3S3) t.dst[1][i] = o1;
    } else if (OP == EW_U2_Q3) {
        double u2 = t.src[0][i], u1 = t.src[1][i], q = t.src[2][i];
        t.dst[0][i] = u2;
        t.dst[1][i] = u2 + q;
        t.dst[2][i] = u1 + q;
    }
}

__device__ __forceinline__ double2 ld2(const double *p, int64_t i) {
    return __ldcs(reinterpret_cast<const double2 *>(p) + i);
}
__device__ __forceinline__ void st2(double *p, int64_t i, double2 v) {
    __stcs(reinterpret_cast<double2 *>(p) + i, v);
}

template <int OP>
__device__ __forceinline__ void ew_vec2(const EwTask &t, int64_t i) {
    // i indexes double2 vectors; the two lanes are independent elements.
    if (OP == EW_FORM_ST) {
        double2 v[8];
#pragma unroll
        for (int k = 0; k < 8; k++) v[k] = ld2(t.src[k], i);
        double o0[8], o1[8];
        form_st(v[0].x, v[1].x, v[2].x, v[3].x, v[4].x, v[5].x, v[6].x, v[7].x, o0);
        form_st(v[0].y, v[1].y, v[2].y, v[3].y, v[4].y, v[5].y, v[6].y, v[7].y, o1);
#pragma unroll
        for (int k = 0; k < 8; k++) st2(t.dst[k], i, make_double2(o0[k], o1[k]));
    } else if (OP == EW_CALC_CIJ) {
        double2 v[7];
#pragma unroll
        for (int k = 0; k < 7; k++) v[k] = ld2(t.src[k], i);
        double q0[7], q1[7], c0[4], c1[4];
#pragma unroll
        for (int k = 0; k < 7; k++) { q0[k] = v[k].x; q1[k] = v[k].y; }
        calc_cij(q0, c0);
        calc_cij(q1, c1);
#pragma unroll
        for (int k = 0; k < 4; k++) st2(t.dst[k], i, make_double2(c0[k], c1[k]));
    } else if (OP == EW_COPY) {
        st2(t.dst[0], i, ld2(t.src[0], i));
    } else if (OP == EW_ADD_DUP) {
        double2 a = ld2(t.src[0], i), b = ld2(t.src[1], i);
        double2 r = make_double2(a.x + b.x, a.y + b.y);
        st2(t.dst[0], i, r);
        st2(t.dst[1], i, r);
    } else if (OP == EW_ADD) {
        double2 a = ld2(t.src[0], i), b = ld2(t.src[1], i);
        st2(t.dst[0], i, make_double2(a.x + b.x, a.y + b.y));
    } else if (OP == EW_SUB) {
        double2 a = ld2(t.src[0], i), b = ld2(t.src[1], i);
        st2(t.dst[0], i, make_double2(a.x - b.x, a.y - b.y));
    } else if (OP == EW_ADD2) {
        double2 a = ld2(t.src[0], i), b = ld2(t.src[1], i), q = ld2(t.src[2], i);
        double2 r0 = make_double2(a.x + q.x, a.y + q.y);
        double2 r1 = make_double2(b.x + q.x, b.y + q.y);
        st2(t.dst[0], i, r0);
        st2(t.dst[1], i, r1);
    } else if (OP >= EW_FORM_T4S4 && OP <= EW_FORM_T6) {
        // only the sources the formula reads are loaded
        double2 v[8];
#pragma unroll
        for (int k = 0; k < 8; k++)
            v[k] = lean_reads<OP>(k) ? ld2(t.src[k], i) : make_double2(0.0, 0.0);
        double a0, a1, b0, b1;
        form_lean<OP>(v[0].x, v[1].x, v[2].x, v[3].x, v[4].x, v[5].x, v[6].x, v[7].x, a0, a1);
        form_lean<OP>(v[0].y, v[1].y, v[2].y, v[3].y, v[4].y, v[5].y, v[6].y, v[7].y, b0, b1);
        st2(t.dst[0], i, make_double2(a0, b0));
        if (OP <= EW_FORM_T3S3) st2(t.dst[1], i, make_double2(a1, b1));
    } else if (OP == EW_U2_Q3) {
        double2 u2 = ld2(t.src[0], i), u1 = ld2(t.src[1], i), q = ld2(t.src[2], i);
        st2(t.dst[0], i, u2);
        st2(t.dst[1], i, make_double2(u2.x + q.x, u2.y + q.y));
        st2(t.dst[2], i, make_double2(u1.x + q.x, u1.y + q.y));
    }
}

template <int OP, bool VEC>
__global__ void __launch_bounds__(256) ew_kernel(const EwTask *__restrict__ tasks, int64_t q) {
    const EwTask t = tasks[blockIdx.y];
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    if (VEC) {
        const int64_t nv = q >> 1;
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += stride)
            ew_vec2<OP>(t, i);
    } else {
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < q; i += stride)
            ew_scalar<OP>(t, i);
    }
}

static int ew_nsrc(int op) {
    switch (op) {
        case EW_FORM_ST: case EW_FORM_T4S4: case EW_FORM_T5S5: case EW_FORM_T3S3: case EW_FORM_S7:
        case EW_FORM_T6: return 8;
        case EW_U2_Q3: return 3;
        case EW_COPY: return 1;
        case EW_ADD_DUP: case EW_ADD: case EW_SUB: return 2;
        case EW_ADD2: return 3;
        case EW_CALC_CIJ: return 7;
    }
    return 0;
}
static int ew_ndst(int op) {
    switch (op) {
        case EW_FORM_ST: return 8;
        case EW_ADD_DUP: case EW_ADD2: case EW_FORM_T4S4: case EW_FORM_T5S5: case EW_FORM_T3S3: return 2;
        case EW_U2_Q3: return 3;
        case EW_CALC_CIJ: return 4;
    }
    return 1;
}
int ew_sources(int op) { return ew_nsrc(op); }
int ew_dests(int op) { return ew_ndst(op); }

template <int OP>
static void launch_op(bool vec, const EwTask *tasks, int count, int64_t q, cudaStream_t s) {
    const int threads = 256;
    int64_t work = vec ? (q >> 1) : q;
    // enough blocks to cover ~4 waves of the 152 SMs across all tasks
    int64_t want = (work + threads - 1) / threads;
    int64_t cap = (int64_t)152 * 8 * 4 / (count > 0 ? count : 1);
    if (cap < 1) cap = 1;
    if (want > cap) want = cap;
    if (want < 1) want = 1;
    dim3 grid((unsigned)want, (unsigned)count);
    if (vec)
        ew_kernel<OP, true><<<grid, threads, 0, s>>>(tasks, q);
    else
        ew_kernel<OP, false><<<grid, threads, 0, s>>>(tasks, q);
}

cudaError_t launch_elementwise(int op, const EwTask *tasks, int count, int64_t q,
                               cudaStream_t stream, bool vec) {
    if (count <= 0 || q <= 0) return cudaSuccess;
    for (int base = 0; base < count; base += 65535) {
        int c = count - base < 65535 ? count - base : 65535;
        const EwTask *t = tasks + base;
        switch (op) {
            case EW_FORM_ST: launch_op<EW_FORM_ST>(vec, t, c, q, stream); break;
            case EW_COPY: launch_op<EW_COPY>(vec, t, c, q, stream); break;
            case EW_ADD_DUP: launch_op<EW_ADD_DUP>(vec, t, c, q, stream); break;
            case EW_ADD: launch_op<EW_ADD>(vec, t, c, q, stream); break;
            case EW_SUB: launch_op<EW_SUB>(vec, t, c, q, stream); break;
            case EW_ADD2: launch_op<EW_ADD2>(vec, t, c, q, stream); break;
            case EW_CALC_CIJ: launch_op<EW_CALC_CIJ>(vec, t, c, q, stream); break;
            case EW_FORM_T4S4: launch_op<EW_FORM_T4S4>(vec, t, c, q, stream); break;
            case EW_FORM_T5S5: launch_op<EW_FORM_T5S5>(vec, t, c, q, stream); break;
            case EW_FORM_T3S3: launch_op<EW_FORM_T3S3>(vec, t, c, q, stream); break;
            case EW_FORM_S7: launch_op<EW_FORM_S7>(vec, t, c, q, stream); break;
            case EW_FORM_T6: launch_op<EW_FORM_T6>(vec, t, c, q, stream); break;
            case EW_U2_Q3: launch_op<EW_U2_Q3>(vec, t, c, q, stream); break;
            default: return cudaErrorInvalidValue;
        }
        count_launch();
    }
    return cudaGetLastError();
}

cudaError_t launch_elementwise(int op, const EwTask *tasks, int count, int64_t q,
                               cudaStream_t stream) {
    return launch_elementwise(op, tasks, count, q, stream, false);
}

// ---------------------------------------------------------------------------
// Layout reorder: column-major n x n  <->  CAPS recursive block layout.
// Restates distributeFrom1ProcRec / collectTo1ProcRec (communication.cpp:
// 612-704) for one rank: nrec quadrant levels (TL, BL, TR, BR = offsets
// 0,1,2,3 x quarter), then bs x bs column-major blocks, blocks column-major.
//
// A block column is a run of bs consecutive doubles in the CAPS layout and
// bs consecutive rows of one column of the column-major matrix: the reorder
// is a copy of n^2 / bs runs.  A warp copies one run (runs of 32 and more:
// the leaf columns when bs is 1 or the leaf, which is the workloads' case),
// with 16-byte accesses when both ends of the run are 16-byte aligned; the
// run's position is worked out once per run from its index (the quadrant
// digits of its leaf, its block and column).  Shorter runs take one thread
// per element.  HBM-bound either way: 16 bytes moved per element.
// ---------------------------------------------------------------------------
struct ReorderGeom {
    int64_t n, m, mm;   // matrix, leaf, leaf^2
    int nrec;
    int bs;             // effective block size (m when bs == 1 or bs == m)
    int nb;             // blocks per leaf side
};

// column-major offset of the first element of run `run` (run = leaf * (mm /
// bs) + blk * bs + cc: block blk of the leaf, column cc of the block)
__device__ __forceinline__ int64_t run_colmajor_offset(const ReorderGeom &g, int64_t run) {
    const int64_t runs_per_leaf = g.mm / g.bs;
    const int64_t leaf = run / runs_per_leaf;
    const int64_t rest = run - leaf * runs_per_leaf;
    int64_t r = 0, c = 0;
    for (int l = 0; l < g.nrec; l++) {
        int d = (int)((leaf >> (2 * (g.nrec - 1 - l))) & 3);
        int64_t h = g.n >> (l + 1);
        r += (d & 1) * h;
        c += (d >> 1) * h;
    }
    const int64_t blk = rest / g.bs, cc = rest - blk * g.bs;
    const int64_t bj = blk % g.nb, bi = blk / g.nb;  // block row, block column
    r += bj * g.bs;
    c += bi * g.bs + cc;
    return r + c * g.n;
}

__device__ __forceinline__ int64_t caps_to_colmajor_index(const ReorderGeom &g, int64_t idx) {
    const int64_t run = idx / g.bs;
    return run_colmajor_offset(g, run) + (idx - run * g.bs);
}

// one warp per run of bs >= 32 doubles
template <bool TO_CAPS>
__device__ __forceinline__ void reorder_runs(const double *__restrict__ s, double *__restrict__ d,
                                             const ReorderGeom &g, int64_t warp0, int64_t nwarps) {
    const int lane = threadIdx.x & 31;
    const int64_t runs = g.n * g.n / g.bs;
    for (int64_t run = warp0; run < runs; run += nwarps) {
        const int64_t cm = run_colmajor_offset(g, run), cp = run * g.bs;
        const double *src = s + (TO_CAPS ? cm : cp);
        double *dst = d + (TO_CAPS ? cp : cm);
        if (((g.bs & 1) == 0) && (((uintptr_t)src | (uintptr_t)dst) & 15) == 0) {
            const double2 *s2 = reinterpret_cast<const double2 *>(src);
            double2 *d2 = reinterpret_cast<double2 *>(dst);
            for (int64_t k = lane; k < g.bs / 2; k += 32) __stcs(d2 + k, __ldcs(s2 + k));
        } else {
            for (int64_t k = lane; k < g.bs; k += 32) __stcs(dst + k, __ldcs(src + k));
        }
    }
}

template <bool TO_CAPS>
__device__ __forceinline__ void reorder_elements(const double *__restrict__ s, double *__restrict__ d,
                                                 const ReorderGeom &g, int64_t t0, int64_t nthreads) {
    const int64_t total = g.n * g.n;
    for (int64_t idx = t0; idx < total; idx += nthreads) {
        int64_t cm = caps_to_colmajor_index(g, idx);
        if (TO_CAPS)
            d[idx] = __ldcs(s + cm);
        else
            d[cm] = __ldcs(s + idx);
    }
}

template <bool TO_CAPS>
__global__ void __launch_bounds__(256) reorder_kernel(const double *const *__restrict__ src,
                                                      double *const *__restrict__ dst,
                                                      ReorderGeom g) {
    const double *s = src[blockIdx.y];
    double *d = dst[blockIdx.y];
    if (g.bs >= 32)
        reorder_runs<TO_CAPS>(s, d, g, ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5,
                              ((int64_t)gridDim.x * blockDim.x) >> 5);
    else
        reorder_elements<TO_CAPS>(s, d, g, (int64_t)blockIdx.x * blockDim.x + threadIdx.x,
                                  (int64_t)gridDim.x * blockDim.x);
}

static ReorderGeom make_geom(int64_t n, int nrec, int64_t bs) {
    ReorderGeom g;
    g.n = n;
    g.nrec = nrec;
    g.m = n >> nrec;
    g.mm = g.m * g.m;
    g.bs = (bs == 1 || bs == g.m) ? (int)g.m : (int)bs;
    g.nb = (int)(g.m / g.bs);
    return g;
}

// grid: enough blocks for a run (or element) per thread, at most 8 blocks of
// 256 threads per SM for all matrices together
static unsigned reorder_blocks(const ReorderGeom &g, int count) {
    const int64_t items = g.bs >= 32 ? g.n * g.n / g.bs * 32 : g.n * g.n;
    int64_t blocks = (items + 255) / 256;
    int64_t cap = (int64_t)152 * 8 / count;
    if (cap < 1) cap = 1;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    return (unsigned)blocks;
}

cudaError_t launch_reorder(const double *const *src_dev, double *const *dst_dev, int count,
                           int64_t n, int nrec, int64_t bs, bool to_caps, cudaStream_t stream) {
    if (count <= 0) return cudaSuccess;
    ReorderGeom g = make_geom(n, nrec, bs);
    dim3 grid(reorder_blocks(g, count), (unsigned)count);
    if (to_caps)
        reorder_kernel<true><<<grid, 256, 0, stream>>>(src_dev, dst_dev, g);
    else
        reorder_kernel<false><<<grid, 256, 0, stream>>>(src_dev, dst_dev, g);
    count_launch();
    return cudaGetLastError();
}

template <bool TO_CAPS>
__global__ void __launch_bounds__(256) reorder_one_kernel(const double *__restrict__ s,
                                                          double *__restrict__ d, ReorderGeom g) {
    if (g.bs >= 32)
        reorder_runs<TO_CAPS>(s, d, g, ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5,
                              ((int64_t)gridDim.x * blockDim.x) >> 5);
    else
        reorder_elements<TO_CAPS>(s, d, g, (int64_t)blockIdx.x * blockDim.x + threadIdx.x,
                                  (int64_t)gridDim.x * blockDim.x);
}

cudaError_t launch_reorder_one(const double *src, double *dst, int64_t n, int nrec, int64_t bs,
                               bool to_caps, cudaStream_t stream) {
    ReorderGeom g = make_geom(n, nrec, bs);
    const unsigned blocks = reorder_blocks(g, 1);
    if (to_caps)
        reorder_one_kernel<true><<<blocks, 256, 0, stream>>>(src, dst, g);
    else
        reorder_one_kernel<false><<<blocks, 256, 0, stream>>>(src, dst, g);
    count_launch();
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Transpose in the recursive layout with bs = 1 (leaves column-major m x m),
// times `sign` (+1 or -1, exact).  X^T has quadrants 11 = X11^T, 21 = X12^T,
// 12 = X21^T, 22 = X22^T at every level, so leaf L of X^T is the transpose
// of the leaf whose base-4 digits are L's with the row and column bit of
// each digit swapped.  One block moves one 32 x 32 tile through shared
// memory, reads and writes both coalesced; grid-stride over (leaf, tile).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) rec_transpose_kernel(const double *__restrict__ s, double *__restrict__ d,
                                                            int64_t m, int64_t leaves, int64_t tside, double sign) {
    __shared__ double tile[32][33];
    const int64_t per_leaf = tside * tside, total = leaves * per_leaf, mm = m * m;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int64_t it = blockIdx.x; it < total; it += gridDim.x) {
        const int64_t leaf = it / per_leaf, t = it - leaf * per_leaf;
        const int64_t ti = t % tside, tj = t / tside;  // destination tile (row, column)
        const uint64_t L = (uint64_t)leaf;
        const int64_t sleaf = (int64_t)(((L & 0x5555555555555555ull) << 1) | ((L >> 1) & 0x5555555555555555ull));
        const double *sl = s + sleaf * mm;
        double *dl = d + leaf * mm;
        // destination (i, j) = source (j, i): tile (ti, tj) reads source rows
        // tj*32.., columns ti*32..; tile[c][r] holds source (tj*32 + r, ti*32 + c)
        for (int k = ty; k < 32; k += 8) {
            const int64_t r = tj * 32 + tx, c = ti * 32 + k;
            if (r < m && c < m) tile[k][tx] = sl[r + c * m];
        }
        __syncthreads();
        for (int k = ty; k < 32; k += 8) {
            const int64_t i = ti * 32 + tx, j = tj * 32 + k;
            if (i < m && j < m) dl[i + j * m] = sign * tile[tx][k];
        }
        __syncthreads();
    }
}

cudaError_t launch_rec_transpose(const double *src, double *dst, int64_t n, int nrec, bool negate,
                                 cudaStream_t stream) {
    const int64_t m = n >> nrec, leaves = (int64_t)1 << (2 * nrec), tside = (m + 31) / 32;
    const int64_t total = leaves * tside * tside;
    const int64_t blocks = total < 152 * 16 ? total : 152 * 16;
    rec_transpose_kernel<<<(unsigned)blocks, 256, 0, stream>>>(src, dst, m, leaves, tside, negate ? -1.0 : 1.0);
    count_launch();
    return cudaGetLastError();
}

// C = alpha * C + P, the product rounded, then the sum (the order of a dgemm
// that scales C by beta before accumulating); alpha = 1 makes the first step
// exact.  16-byte aligned pointers take two elements per load.
template <bool VEC>
__global__ void __launch_bounds__(256) scale_add_kernel(double *__restrict__ c, const double *__restrict__ p,
                                                        double alpha, int64_t count) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    if (VEC) {
        double2 *c2 = reinterpret_cast<double2 *>(c);
        const double2 *p2 = reinterpret_cast<const double2 *>(p);
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count / 2; i += stride) {
            double2 x = c2[i];
            const double2 y = __ldcs(p2 + i);
            x.x = __dadd_rn(__dmul_rn(alpha, x.x), y.x);
            x.y = __dadd_rn(__dmul_rn(alpha, x.y), y.y);
            c2[i] = x;
        }
    } else {
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride)
            c[i] = __dadd_rn(__dmul_rn(alpha, c[i]), __ldcs(p + i));
    }
}

cudaError_t launch_scale_add(double *c, const double *p, double alpha, int64_t count, cudaStream_t stream) {
    if (count <= 0) return cudaSuccess;
    const bool vec = (((uintptr_t)c | (uintptr_t)p) & 15) == 0 && count % 2 == 0;
    const int64_t work = vec ? count / 2 : count;
    int64_t blocks = (work + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (vec)
        scale_add_kernel<true><<<(unsigned)blocks, 256, 0, stream>>>(c, p, alpha, count);
    else
        scale_add_kernel<false><<<(unsigned)blocks, 256, 0, stream>>>(c, p, alpha, count);
    count_launch();
    return cudaGetLastError();
}

}  // namespace caps
