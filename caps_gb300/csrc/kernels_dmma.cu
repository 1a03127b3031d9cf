// Plain form base case: C = A * B on FP64 DMMA tensor cores (mma.sync f64).
//
// Replaces block_multiply -> square_dgemm_zero -> dgemm_ (multiply.cpp:
// 1082-1141, dgemm-blas.cpp:4-13): column-major m x m operands, beta = 0.
//
// GB300 runs FP64 (DFMA and DMMA alike) at ~1.05 TFLOP/s for the whole GPU,
// about 1.8 multiply-adds per clock per SM, so this kernel is bound by the
// DMMA pipe at any sensible tiling; 64x64 tiles with a 16-deep K slab in
// shared memory keep operand traffic far below what that pipe can consume.
// One CTA (4 warps, 2x2, 32x32 per warp of m8n8k4 tiles) per 64x64 tile of
// one leaf of the batch (blockIdx.z).
#include "common.cuh"

namespace caps {

namespace {
constexpr int BM = 64, BN = 64, BK = 16, LDS = 72;  // LDS: padded row (banks)

__device__ __forceinline__ void dmma_8x8x4(double (&d)[2], double a, double b) {
    asm volatile(
        "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
        : "+d"(d[0]), "+d"(d[1])
        : "d"(a), "d"(b));
}
}  // namespace

__global__ void __launch_bounds__(128) dmma_gemm_kernel(const LeafTask *__restrict__ tasks, int m) {
    __shared__ double As[BK][LDS];  // As[k][i]
    __shared__ double Bs[BK][LDS];  // Bs[k][j]
    const LeafTask t = tasks[blockIdx.z];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wr = warp >> 1, wc = warp & 1;
    const int64_t i0 = (int64_t)blockIdx.y * BM, j0 = (int64_t)blockIdx.x * BN;
    const int64_t M = m;

    double acc[4][4][2];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b][0] = acc[a][b][1] = 0.0;

    for (int64_t k0 = 0; k0 < M; k0 += BK) {
        // A tile: 64 rows x 16 k, column-major source; thread -> (row, k pair)
#pragma unroll
        for (int p = 0; p < 8; p++) {
            int row = tid & 63, kk = (tid >> 6) + 2 * p;
            int64_t gi = i0 + row, gk = k0 + kk;
            As[kk][row] = (gi < M && gk < M) ? t.A[gi + gk * M] : 0.0;
        }
        // B tile: 16 k x 64 cols; thread -> (k, col)
#pragma unroll
        for (int p = 0; p < 8; p++) {
            int kk = tid & 15, col = (tid >> 4) + 8 * p;
            int64_t gk = k0 + kk, gj = j0 + col;
            Bs[kk][col] = (gk < M && gj < M) ? t.B[gk + gj * M] : 0.0;
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
                int64_t gi = i0 + 32 * wr + 8 * a + (lane >> 2);
                int64_t gj = j0 + 32 * wc + 8 * b + 2 * (lane & 3) + e;
                if (gi < M && gj < M) t.C[gi + gj * M] = acc[a][b][e];
            }
}

cudaError_t launch_dmma_gemm(const LeafTask *tasks_dev, int count, int m, cudaStream_t stream) {
    if (count <= 0 || m <= 0) return cudaSuccess;
    unsigned tiles = (unsigned)((m + BM - 1) / BM);
    for (int base = 0; base < count; base += 65535) {
        int c = count - base < 65535 ? count - base : 65535;
        dim3 grid(tiles, tiles, (unsigned)c);
        dmma_gemm_kernel<<<grid, 128, 0, stream>>>(tasks_dev + base, m);
        count_launch();
    }
    return cudaGetLastError();
}

}  // namespace caps
