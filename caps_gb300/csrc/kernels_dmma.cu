// Plain form base case: C = A * B on FP64 DMMA tensor cores (mma.sync f64).
//
// Replaces block_multiply -> square_dgemm_zero -> dgemm_ (multiply.cpp:
// 1082-1141, dgemm-blas.cpp:4-13): column-major m x m operands, beta = 0;
// and the rectangular subproject's base case localRectMM (rect-class/
// rectmm.cpp:47-51): A m x k, B k x n, C m x n, column-major, beta = 0.
//
// GB300 runs FP64 (DFMA and DMMA alike) at ~1.05 TFLOP/s for the whole GPU,
// about 1.8 multiply-adds per clock per SM, so this kernel is bound by the
// DMMA pipe at any sensible tiling; a 16-deep K slab in shared memory keeps
// operand traffic far below what that pipe can consume.  Each warp owns a
// 32 x 32 block of C (4 x 4 m8n8k4 tiles); a CTA is a WM x WN grid of warps,
// one CTA per (32 WM) x (32 WN) tile of one leaf of the batch (blockIdx.z).
// Three shapes (caps_dmma_tile): 64 x 64 (2 x 2 warps, the default),
// 32 x 32 (one warp: four times the CTAs, for small leaves) and 128 x 64
// (4 x 2 warps: half the B traffic per multiply-add).  The autotuner times
// them per size.  The epilogue applies the task's fold (DmmaFold) of the
// lean 'd' step that consumes the product.
#include "common.cuh"

namespace caps {

namespace {
constexpr int BK = 16;

__device__ __forceinline__ void dmma_8x8x4(double (&d)[2], double a, double b) {
    asm volatile(
        "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
        : "+d"(d[0]), "+d"(d[1])
        : "d"(a), "d"(b));
}
}  // namespace

template <int WM, int WN>
__global__ void __launch_bounds__(32 * WM * WN) dmma_gemm_kernel(const DmmaTask *__restrict__ tasks, int m, int n,
                                                                 int k) {
    constexpr int BM = 32 * WM, BN = 32 * WN, NT = 32 * WM * WN;
    constexpr int LDA = BM + 8, LDB = BN + 8;  // padded rows (banks)
    __shared__ double As[BK][LDA];  // As[k][i]
    __shared__ double Bs[BK][LDB];  // Bs[k][j]
    const DmmaTask t = tasks[blockIdx.z];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wr = warp / WN, wc = warp % WN;
    const int64_t i0 = (int64_t)blockIdx.y * BM, j0 = (int64_t)blockIdx.x * BN;
    const int64_t M = m, N = n, K = k;  // A: M x K, B: K x N, C: M x N

    double acc[4][4][2];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b][0] = acc[a][b][1] = 0.0;

    for (int64_t k0 = 0; k0 < K; k0 += BK) {
        // A tile: BM rows x 16 k from a column-major source; consecutive
        // threads read consecutive rows of one column
#pragma unroll
        for (int p = 0; p < BM * BK / NT; p++) {
            const int e = tid + NT * p, row = e % BM, kk = e / BM;
            const int64_t gi = i0 + row, gk = k0 + kk;
            As[kk][row] = (gi < M && gk < K) ? t.A[gi + gk * M] : 0.0;
        }
        // B tile: 16 k x BN columns; consecutive threads read the 16 k of one column
#pragma unroll
        for (int p = 0; p < BN * BK / NT; p++) {
            const int e = tid + NT * p, kk = e % BK, col = e / BK;
            const int64_t gk = k0 + kk, gj = j0 + col;
            Bs[kk][col] = (gk < K && gj < N) ? t.B[gk + gj * K] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < BK; ks += 4) {
            double af[4], bf[4];
#pragma unroll
            for (int a = 0; a < 4; a++) af[a] = As[ks + (lane & 3)][32 * wr + 8 * a + (lane >> 2)];
#pragma unroll
            for (int b = 0; b < 4; b++) bf[b] = Bs[ks + (lane & 3)][32 * wc + 8 * b + (lane >> 2)];
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int b = 0; b < 4; b++) dmma_8x8x4(acc[a][b], af[a], bf[b]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++)
#pragma unroll
            for (int e = 0; e < 2; e++) {
                const int64_t gi = i0 + 32 * wr + 8 * a + (lane >> 2);
                const int64_t gj = j0 + 32 * wc + 8 * b + 2 * (lane & 3) + e;
                if (gi >= M || gj >= N) continue;
                const int64_t x = gi + gj * M;
                const double p = acc[a][b][e];
                switch (t.fold) {
                    case FOLD_ADD: t.C[x] = t.s0[x] + p; break;
                    case FOLD_SUB: t.C[x] = t.s0[x] - p; break;
                    case FOLD_ADD_DUP: {
                        const double v = t.s0[x] + p;
                        t.C[x] = v;
                        t.d1[x] = v;
                        break;
                    }
                    case FOLD_U2_Q3: {
                        const double u2 = t.s0[x], u1 = t.s1[x];
                        t.C[x] = u2;
                        t.d1[x] = u2 + p;
                        t.d2[x] = u1 + p;
                        break;
                    }
                    default: t.C[x] = p;
                }
            }
}

template <int WM, int WN>
static cudaError_t launch_dmma_shape(const DmmaTask *tasks_dev, int count, int m, int n, int k, cudaStream_t stream) {
    const unsigned rows = (unsigned)((m + 32 * WM - 1) / (32 * WM)), cols = (unsigned)((n + 32 * WN - 1) / (32 * WN));
    for (int base = 0; base < count; base += 65535) {
        const int c = count - base < 65535 ? count - base : 65535;
        dim3 grid(cols, rows, (unsigned)c);
        dmma_gemm_kernel<WM, WN><<<grid, 32 * WM * WN, 0, stream>>>(tasks_dev + base, m, n, k);
        count_launch();
    }
    return cudaGetLastError();
}

void dmma_tile_shape(int tile, int *rows, int *cols) {
    switch (tile) {
        case DMMA_TILE_32x32: *rows = 32; *cols = 32; break;
        case DMMA_TILE_128x64: *rows = 128; *cols = 64; break;
        default: *rows = 64; *cols = 64; break;
    }
}

cudaError_t launch_dmma_rect(const DmmaTask *tasks_dev, int count, int m, int n, int k, cudaStream_t stream,
                             int tile) {
    if (count <= 0 || m <= 0 || n <= 0) return cudaSuccess;
    switch (tile) {
        case DMMA_TILE_32x32: return launch_dmma_shape<1, 1>(tasks_dev, count, m, n, k, stream);
        case DMMA_TILE_128x64: return launch_dmma_shape<4, 2>(tasks_dev, count, m, n, k, stream);
        default: return launch_dmma_shape<2, 2>(tasks_dev, count, m, n, k, stream);
    }
}

cudaError_t launch_dmma_gemm(const DmmaTask *tasks_dev, int count, int m, cudaStream_t stream, int tile) {
    return launch_dmma_rect(tasks_dev, count, m, m, m, stream, tile);
}

}  // namespace caps
