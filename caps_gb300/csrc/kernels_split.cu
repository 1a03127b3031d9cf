// Split form of the base case (Ozaki-style), on tcgen05 tensor cores.
//
// The reference multiplies leaves with FP64 dgemm (multiply.cpp:1124,
// dgemm-blas.cpp:4-13).  Here each leaf product C = A * B (column-major m x m)
// is computed as follows:
//
//  1. scan:     per row i of A the exponent bound E (|a_ij| < 2^E) and the
//               lowest set bit; the same per column of B.
//  2. finalize: f_i = 55 - E_i; digits needed = ceil((E - lsb + 1) / 7),
//               max over the launch group (exact for integer-like inputs).
//  3. slice:    X = round(a * 2^f) (|X| <= 2^55) is cut into balanced base-128
//               digits d_1..d_8 (|d| <= 64), the s most significant kept.
//               Digits are int8 values carried EXACTLY in bf16, written as
//               pre-tiled UMMA canonical K-major tiles (no swizzle): 8-row x
//               16-byte core matrices, the two K halves of a row group side
//               by side (K stride 128 B, row-group stride 256 B), one plane
//               after another (A: 128 x 16 = 4 KiB, B: 64 x 16 = 2 KiB).
//  4. gemm:     every digit pair (a, b) with a + b <= nd + 1 is multiplied on
//               tcgen05.mma kind::f16 (bf16 x bf16 -> f32).  Pairs of one
//               diagonal t = a + b share one TMEM accumulator (64 columns):
//               products are <= 2^12, a diagonal has <= 8 pairs, so 512-deep
//               K chunks sum to <= 2^24 and stay EXACT in fp32.  After each
//               chunk the epilogue warps move the diagonals into exact int64
//               sums hi = sum_{t<=5} c_t 2^{7(5-t)}, lo = sum_{t>=6} c_t
//               2^{7(9-t)}, and at the end C = (hi 2^28 + lo) 2^{49-f_i-g_j}
//               with one FP64 rounding.
//
// GB300 (sm_103a) has no tcgen05 kind::i8, and its FP64 pipe is ~1 TFLOP/s,
// so the integer slice products go to the bf16 tensor pipe (exact for these
// ranges) and FP64 work stays O(1) per output element.
//
// Each MMA multiplies one A digit plane (128 x 16) by up to four B planes
// concatenated along N (N = 64 x planes <= 256), writing four consecutive
// diagonals at once: 12 MMAs per 16-deep K step for s = nd = 8.
//
// All mbarrier waits are bounded; a wait that gives up sets a bit in the
// status word the host reads back (CAPS_ERR_TIMEOUT) and the kernel unwinds,
// waiting (bounded) for its own copies and MMAs before freeing TMEM.
#include "split_common.cuh"

namespace caps {

using namespace split;

namespace {

constexpr int CHUNK = 32;       // K16 steps per exact accumulation chunk (K = 512)
constexpr int SUB = 2;           // 16-deep K steps per pipeline stage (K = 32 per stage)
constexpr int NSTAGE = 2;
constexpr int A_PLANE_BYTES = TM * TK * 2;  // 4096
constexpr int B_PLANE_BYTES = TN * TK * 2;  // 2048
constexpr int STAGE_A = SUB * MAXS * A_PLANE_BYTES;
constexpr int STAGE_B = SUB * MAXS * B_PLANE_BYTES;
constexpr int STAGE_BYTES = STAGE_A + STAGE_B;  // 96 KiB
constexpr int GEMM_THREADS = 320;               // producer, MMA, 8 epilogue warps

}  // namespace

size_t split_workspace_bytes(int m, int count, int scheme) {
    return make_geo(m, count, scheme).total;
}

// ---------------------------------------------------------------- scan
// Per row of A and per column of B: the largest exponent and the lowest set
// bit over the leaf.  Work units of up to 64K elements each, the same on both
// sides: grid.y = 0, a block of A rows (512, a thread per two adjacent rows)
// times a slab of 128 columns; grid.y = 1, a block of 32 B columns (a warp
// per 4 columns).  16-byte loads when the leaf's element pairs are 16-byte
// aligned (m even, base aligned), 8-byte loads otherwise.  grid.x strides
// over (leaf, unit).
constexpr int SCAN_AROWS = 512, SCAN_KSLAB = 128, SCAN_BCOLS = 32;

__device__ __forceinline__ void scan_value(double x, int &emax, int &lmin) {
    if (nonzero_bits(x)) {
        int E, lb;
        exp_lsb(x, E, lb);
        emax = E > emax ? E : emax;
        lmin = lb < lmin ? lb : lmin;
    }
}

__device__ __forceinline__ int64_t scan_units(int64_t M) {
    const int64_t a = ((M + SCAN_AROWS - 1) / SCAN_AROWS) * ((M + SCAN_KSLAB - 1) / SCAN_KSLAB);
    const int64_t b = (M + SCAN_BCOLS - 1) / SCAN_BCOLS;
    return a > b ? a : b;
}

__global__ void __launch_bounds__(256) split_scan_kernel(const LeafTask *__restrict__ tasks,
                                                         char *__restrict__ ws, Geo g) {
    const int64_t M = g.m, per = scan_units(M), total = per * g.count;
    const int64_t rowblocks = (M + SCAN_AROWS - 1) / SCAN_AROWS;
    const int64_t aunits = rowblocks * ((M + SCAN_KSLAB - 1) / SCAN_KSLAB);
    const int64_t bunits = (M + SCAN_BCOLS - 1) / SCAN_BCOLS;
    for (int64_t it = blockIdx.x; it < total; it += gridDim.x) {
        const int l = (int)(it / per);
        const int64_t u = it - (int64_t)l * per;
        const LeafTask t = tasks[l];
        char *sc = leaf_scalars(ws, g, l);
        if (blockIdx.y == 0) {
            if (u >= aunits) continue;
            const int64_t i0 = (u % rowblocks) * SCAN_AROWS + 2 * threadIdx.x;
            const int64_t k0 = (u / rowblocks) * SCAN_KSLAB;
            const int64_t k1 = k0 + SCAN_KSLAB < M ? k0 + SCAN_KSLAB : M;
            if (i0 >= M) continue;
            int e0 = -100000, l0 = 100000, e1 = -100000, l1 = 100000;
            if ((M & 1) == 0 && ((uintptr_t)t.A & 15) == 0) {  // i0 even, M even: the pair is 16-byte aligned
#pragma unroll 8
                for (int64_t k = k0; k < k1; k++) {
                    const double2 v = __ldg(reinterpret_cast<const double2 *>(t.A + i0 + k * M));
                    scan_value(v.x, e0, l0);
                    scan_value(v.y, e1, l1);
                }
            } else {
                const bool two = i0 + 1 < M;
#pragma unroll 8
                for (int64_t k = k0; k < k1; k++) {
                    scan_value(__ldg(t.A + i0 + k * M), e0, l0);
                    if (two) scan_value(__ldg(t.A + i0 + 1 + k * M), e1, l1);
                }
            }
            int *ea = reinterpret_cast<int *>(sc + g.off_ea), *la = reinterpret_cast<int *>(sc + g.off_la);
            if (e0 > -100000) {
                atomicMax(ea + i0, e0 + 4096);
                atomicMax(la + i0, 4096 - l0);
            }
            if (e1 > -100000) {
                atomicMax(ea + i0 + 1, e1 + 4096);
                atomicMax(la + i0 + 1, 4096 - l1);
            }
        } else {
            if (u >= bunits) continue;
            const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
            const bool vec = (M & 1) == 0 && ((uintptr_t)t.B & 15) == 0;
#pragma unroll 1
            for (int c = 0; c < 4; c++) {
                const int64_t j = u * SCAN_BCOLS + w * 4 + c;
                if (j >= M) break;
                const double *col = t.B + j * M;
                int emax = -100000, lmin = 100000;
                if (vec) {
#pragma unroll 8
                    for (int64_t k = 2 * lane; k < M; k += 64) {
                        const double2 v = __ldg(reinterpret_cast<const double2 *>(col + k));
                        scan_value(v.x, emax, lmin);
                        scan_value(v.y, emax, lmin);
                    }
                } else {
#pragma unroll 8
                    for (int64_t k = lane; k < M; k += 32) scan_value(__ldg(col + k), emax, lmin);
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, o));
                    lmin = min(lmin, __shfl_xor_sync(0xffffffffu, lmin, o));
                }
                if (lane == 0 && emax > -100000) {
                    reinterpret_cast<int *>(sc + g.off_eb)[j] = emax + 4096;
                    reinterpret_cast<int *>(sc + g.off_lb)[j] = 4096 - lmin;
                }
            }
        }
    }
}

// f = 55 - E per row / column (digit scheme); digits needed, and the bits
// E - lsb + 1 per side (max over the group) for the scheme choice
__global__ void __launch_bounds__(256) split_finalize_kernel(char *__restrict__ ws, Geo g) {
    char *leaf = leaf_scalars(ws, g, blockIdx.y);
    SplitHdr *h = reinterpret_cast<SplitHdr *>(ws);
    int idx = blockIdx.x * 256 + threadIdx.x;
    int need = 0, bits[2] = {0, 0};
    if (idx < g.m) {
        for (int side = 0; side < 2; side++) {
            int ee = reinterpret_cast<int *>(leaf + (side ? g.off_eb : g.off_ea))[idx];
            int le = reinterpret_cast<int *>(leaf + (side ? g.off_lb : g.off_la))[idx];
            int f = 0;
            if (ee != 0) {
                int E = ee - 4096, lsb = 4096 - le;
                f = 55 - E;
                int b = E - lsb + 1;
                int s = (b + 6) / 7;
                need = s > need ? s : need;
                bits[side] = b;
            }
            reinterpret_cast<int *>(leaf + (side ? g.off_fb : g.off_fa))[idx] = f;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        need = max(need, __shfl_xor_sync(0xffffffffu, need, o));
        bits[0] = max(bits[0], __shfl_xor_sync(0xffffffffu, bits[0], o));
        bits[1] = max(bits[1], __shfl_xor_sync(0xffffffffu, bits[1], o));
    }
    if ((threadIdx.x & 31) == 0) {
        if (need > 0) atomicMax(&h->needed, need);
        if (bits[0] > 0) atomicMax(&h->bitsA, bits[0]);
        if (bits[1] > 0) atomicMax(&h->bitsB, bits[1]);
    }
}

// ---------------------------------------------------------------- slice
// balanced base-128 digits of round(x 2^f), most significant first.
// X + 64 (1 + 128 + ... + 128^7) has ordinary base-128 digits d_k + 64, so
// each balanced digit is a 7-bit field minus 64; the top field is not masked
// (it may reach 128: d_1 = 64 when |X| = 2^55).  Same digits as peeling
// them off one by one with a carry.
__device__ __forceinline__ void digits8(double x, int f, int (&d)[8]) {
    const unsigned long long OFF = 0x0081020408102040ull;  // 64 * sum_{k<8} 128^k
    const unsigned long long U = (unsigned long long)scaled_round(x, f) + OFF;
    const uint32_t lo = (uint32_t)U, hi = (uint32_t)(U >> 32);
    d[7] = (int)(lo & 127u) - 64;
    d[6] = (int)((lo >> 7) & 127u) - 64;
    d[5] = (int)((lo >> 14) & 127u) - 64;
    d[4] = (int)((lo >> 21) & 127u) - 64;
    d[3] = (int)(__funnelshift_r(lo, hi, 28) & 127u) - 64;
    d[2] = (int)((hi >> 3) & 127u) - 64;
    d[1] = (int)((hi >> 10) & 127u) - 64;
    d[0] = (int)(hi >> 17) - 64;
}

// |d| <= 64 has at most 7 significant bits: 1.5 * 2^23 + d is exact in fp32,
// and the top half of the fp32 encoding of d is its exact bf16 encoding
__device__ __forceinline__ uint32_t bf16_of_digit(int d) {
    return __float_as_uint(__int_as_float(0x4B400000 + d) - 12582912.0f) >> 16;
}

// A side: one thread = one row x 8 k (16 bytes per plane); 256 threads = one
// 128 x 16 tile.  B side: one thread = one column x 8 k; 256 threads = two
// 64 x 16 tiles.
__device__ __forceinline__ void split_slice_tile(const LeafTask *__restrict__ tasks, int m, char *__restrict__ ws,
                                                 const Geo &g, int s, int leaf, int64_t tile, int side) {
    const LeafTask t = tasks[leaf];
    char *sc = leaf_scalars(ws, g, leaf);
    char *dg = leaf_digits(ws, g, leaf);
    const int64_t M = m;
    const int tid = threadIdx.x;
    const int64_t atiles = (int64_t)g.mtiles * g.nks;
    if (side == 0) {
        if (tile >= atiles) return;
        int mt = (int)(tile / g.nks), ks = (int)(tile % g.nks);
        int r = tid & 127, kg = tid >> 7;
        int64_t i = (int64_t)mt * TM + r;
        int64_t k0 = (int64_t)ks * TK + kg * 8;
        int f = i < M ? reinterpret_cast<const int *>(sc + g.off_fa)[i] : 0;
        uint32_t packed[MAXS][4];
#pragma unroll
        for (int pl = 0; pl < MAXS; pl++)
#pragma unroll
            for (int q = 0; q < 4; q++) packed[pl][q] = 0;
#pragma unroll
        for (int e = 0; e < 8; e++) {
            int64_t k = k0 + e;
            double x = (i < M && k < M) ? t.A[i + k * M] : 0.0;
            int d[8];
            digits8(x, f, d);
#pragma unroll
            for (int pl = 0; pl < MAXS; pl++) packed[pl][e >> 1] |= bf16_of_digit(d[pl]) << (16 * (e & 1));
        }
        char *base = dg + g.off_da + (size_t)(mt * g.nks + ks) * s * A_PLANE_BYTES;
        size_t off = (size_t)(r >> 3) * 256 + (size_t)kg * 128 + (size_t)(r & 7) * 16;
        for (int pl = 0; pl < s; pl++)
            *reinterpret_cast<uint4 *>(base + (size_t)pl * A_PLANE_BYTES + off) =
                make_uint4(packed[pl][0], packed[pl][1], packed[pl][2], packed[pl][3]);
    } else {
        int64_t btiles = (int64_t)g.ntiles * g.nks;
        int64_t bt = tile * 2 + (tid >> 7);
        if (bt >= btiles) return;
        int nt = (int)(bt / g.nks), ks = (int)(bt % g.nks);
        int c = tid & 63, kg = (tid >> 6) & 1;
        int64_t j = (int64_t)nt * TN + c;
        int64_t k0 = (int64_t)ks * TK + kg * 8;
        int f = j < M ? reinterpret_cast<const int *>(sc + g.off_fb)[j] : 0;
        uint32_t packed[MAXS][4];
#pragma unroll
        for (int pl = 0; pl < MAXS; pl++)
#pragma unroll
            for (int q = 0; q < 4; q++) packed[pl][q] = 0;
#pragma unroll
        for (int e = 0; e < 8; e++) {
            int64_t k = k0 + e;
            double x = (j < M && k < M) ? t.B[k + j * M] : 0.0;
            int d[8];
            digits8(x, f, d);
#pragma unroll
            for (int pl = 0; pl < MAXS; pl++) packed[pl][e >> 1] |= bf16_of_digit(d[pl]) << (16 * (e & 1));
        }
        char *base = dg + g.off_db + (size_t)(nt * g.nks + ks) * s * B_PLANE_BYTES;
        for (int pl = 0; pl < s; pl++) {
            size_t off = (size_t)pl * B_PLANE_BYTES + (size_t)(c >> 3) * 256 + (size_t)kg * 128 +
                         (size_t)(c & 7) * 16;
            *reinterpret_cast<uint4 *>(base + off) =
                make_uint4(packed[pl][0], packed[pl][1], packed[pl][2], packed[pl][3]);
        }
    }
}

// Grid-stride over (leaf, tile), so that the launch is cheap when the residue
// scheme runs and this kernel returns at once.  blockIdx.y: A (0) or B (1).
__global__ void __launch_bounds__(256) split_slice_kernel(const LeafTask *__restrict__ tasks, int m,
                                                          char *__restrict__ ws, Geo g, SplitParams p) {
    const SplitHdr *h = reinterpret_cast<const SplitHdr *>(ws);
    if (h->residues) return;  // the residue scheme runs
    int s, nd;
    resolve_sd(h, p, s, nd);
    const int64_t atiles = (int64_t)g.mtiles * g.nks, btiles2 = ((int64_t)g.ntiles * g.nks + 1) / 2;
    const int64_t per = atiles > btiles2 ? atiles : btiles2;
    const int64_t total = per * g.count;
    for (int64_t it = blockIdx.x; it < total; it += gridDim.x)
        split_slice_tile(tasks, m, ws, g, s, (int)(it / per), it % per, blockIdx.y);
}

// ---------------------------------------------------------------- gemm
namespace {

// The MMA sequence of one 16-deep K step depends only on (s, nd) and on the
// stage: it is built once per CTA (stage 0 addresses), kept in registers, and
// each step adds the stage offset to the descriptors' address fields.
// Recomputing descriptors per MMA in the single issuing thread halved the
// tensor pipe's throughput.  At most 12 MMAs per step for s, nd <= 8.
constexpr int MAX_MMA = 12;

struct MmaTable {
    uint64_t ad[MAX_MMA], bd[MAX_MMA];
    uint32_t id[MAX_MMA], col[MAX_MMA];
    uint32_t fresh;  // bit q: MMA q is the first writer of its regions in a chunk
    int count;
};

__device__ void build_mma_table(MmaTable *t, uint32_t a0, uint32_t b0, int s, int nd) {
    int q = 0, init_hi = -1;
    t->fresh = 0;
    for (int a = 1; a <= s; a++) {
        int jmax = s < nd + 1 - a ? s : nd + 1 - a;
        if (jmax < 1) break;
        int rlo = a - 1, rhi = a - 1 + jmax - 1;
        for (int part = 0; part < 2; part++) {
            // part 0: regions already written this chunk (accumulate);
            // part 1: regions this plane writes first (overwrite on a chunk's first step)
            int ra = part == 0 ? rlo : (rlo > init_hi + 1 ? rlo : init_hi + 1);
            int rb = part == 0 ? (rhi < init_hi ? rhi : init_hi) : rhi;
            for (int r = ra; r <= rb && q < MAX_MMA; r += 4) {
                int cnt = rb - r + 1 < 4 ? rb - r + 1 : 4;
                int j0 = r - (a - 1) + 1;
                // K-direction core-matrix stride (LBO) 128 B, M/N-direction (SBO) 256 B
                t->ad[q] = sdesc(a0 + (uint32_t)(a - 1) * A_PLANE_BYTES, 128, 256);
                t->bd[q] = sdesc(b0 + (uint32_t)(j0 - 1) * B_PLANE_BYTES, 128, 256);
                t->id[q] = idesc_bf16(TM, TN * cnt);
                t->col[q] = (uint32_t)(TN * r);
                if (part == 1) t->fresh |= 1u << q;
                q++;
            }
        }
        if (rhi > init_hi) init_hi = rhi;
    }
    t->count = q;
}

}  // namespace

__global__ void __launch_bounds__(GEMM_THREADS, 1)
    split_gemm_kernel(const LeafTask *__restrict__ tasks, int count, char *__restrict__ ws, Geo g,
                      SplitParams p, unsigned *__restrict__ status, int starve) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char *stA = smem;                      // NSTAGE x STAGE_A
    unsigned char *stB = smem + NSTAGE * STAGE_A;   // NSTAGE x STAGE_B
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + NSTAGE * STAGE_BYTES);
    // bars: full[NSTAGE], empty[NSTAGE], tfull, tempty, final
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * NSTAGE + 3);
    MmaTable *mtab = reinterpret_cast<MmaTable *>(bars + 16);

    if (reinterpret_cast<const SplitHdr *>(ws)->residues) return;  // the residue scheme runs
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // starve (test hook): no copies are issued, so nothing is ever in flight
    // and every wait may give up after a short spin
    const uint32_t wl = starve ? WAIT_LIMIT_STARVED : WAIT_LIMIT;
    int s, nd;
    resolve_sd(reinterpret_cast<const SplitHdr *>(ws), p, s, nd);
    const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + NSTAGE);
    const uint32_t tfull = smem_u32(bars + 2 * NSTAGE), tempty = smem_u32(bars + 2 * NSTAGE + 1);
    const uint32_t finalb = smem_u32(bars + 2 * NSTAGE + 2);

    if (threadIdx.x == 0) {
        for (int i = 0; i < NSTAGE; i++) {
            mbar_init(full0 + 8 * i, 1);
            mbar_init(empty0 + 8 * i, 1);
        }
        mbar_init(tfull, 1);
        mbar_init(tempty, 8);
        mbar_init(finalb, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(
                         smem_u32(tmem_slot))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    const int64_t tiles_per_leaf = (int64_t)g.mtiles * g.ntiles;
    const int64_t total = tiles_per_leaf * count;
    const uint32_t bytesA = (uint32_t)s * A_PLANE_BYTES, bytesB = (uint32_t)s * B_PLANE_BYTES;
    const int nchunks = (g.nks + CHUNK - 1) / CHUNK;

    if (warp == 0) {
        // ------------------------------------------------ producer
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            bool ok = true;
            uint32_t armed[NSTAGE] = {0, 0};  // 1 + phase of the last arm
            for (int64_t tile = blockIdx.x; tile < total && ok && !starve; tile += gridDim.x) {
                int leafi = (int)(tile / tiles_per_leaf);
                int64_t rem = tile % tiles_per_leaf;
                int mt = (int)(rem / g.ntiles), nt = (int)(rem % g.ntiles);
                const char *dg = leaf_digits(ws, g, leafi);
                const char *srcA = dg + g.off_da + (size_t)mt * g.nks * bytesA;
                const char *srcB = dg + g.off_db + (size_t)nt * g.nks * bytesB;
                for (int ch = 0; ch < nchunks && ok; ch++) {
                    const int ks0 = ch * CHUNK, ks1 = ks0 + CHUNK < g.nks ? ks0 + CHUNK : g.nks;
                    for (int ks = ks0; ks < ks1; ks += SUB) {
                        // SUB consecutive 16-deep tiles are adjacent in global memory
                        const uint32_t nsub = ks + SUB <= ks1 ? SUB : (uint32_t)(ks1 - ks);
                        if (!mbar_wait(empty0 + 8 * stage, phase ^ 1, status, 1u, wl)) { ok = false; break; }
                        mbar_expect_tx(full0 + 8 * stage, nsub * (bytesA + bytesB));
                        bulk_g2s(smem_u32(stA + stage * STAGE_A), srcA + (size_t)ks * bytesA, nsub * bytesA,
                                 full0 + 8 * stage);
                        bulk_g2s(smem_u32(stB + stage * STAGE_B), srcB + (size_t)ks * bytesB, nsub * bytesB,
                                 full0 + 8 * stage);
                        armed[stage] = 1 + phase;
                        if (++stage == NSTAGE) { stage = 0; phase ^= 1; }
                    }
                }
            }
            // drain: every armed stage's copies must land before exit
            for (int i = 0; i < NSTAGE; i++)
                if (armed[i]) mbar_wait(full0 + 8 * i, armed[i] - 1, status, 2u, wl);
        }
    } else if (warp == 1) {
        // ------------------------------------------------ MMA issuer
        if (lane == 0) {
            build_mma_table(mtab, smem_u32(stA), smem_u32(stB), s, nd);
            uint64_t tad[MAX_MMA], tbd[MAX_MMA];
            uint32_t tid[MAX_MMA], tcol[MAX_MMA];
#pragma unroll
            for (int q = 0; q < MAX_MMA; q++) {
                tad[q] = mtab->ad[q];
                tbd[q] = mtab->bd[q];
                tid[q] = mtab->id[q];
                tcol[q] = tmem + mtab->col[q];
            }
            const uint32_t tfresh = mtab->fresh;
            const int nmma = mtab->count;
            int stage = 0;
            uint32_t phase = 0, chunk_ctr = 0;
            bool ok = true;
            for (int64_t tile = blockIdx.x; tile < total && ok; tile += gridDim.x) {
                for (int ch = 0; ch < nchunks && ok; ch++) {
                    if (!mbar_wait(tempty, (chunk_ctr & 1) ^ 1, status, 4u, wl)) { ok = false; break; }
                    tc_fence_after();
                    int ks0 = ch * CHUNK, ks1 = ks0 + CHUNK < g.nks ? ks0 + CHUNK : g.nks;
                    for (int ks = ks0; ks < ks1; ks += SUB) {
                        const int nsub = ks + SUB <= ks1 ? SUB : ks1 - ks;
                        if (!mbar_wait(full0 + 8 * stage, phase, status, 8u, wl)) { ok = false; break; }
                        tc_fence_after();
#pragma unroll
                        for (int sub = 0; sub < SUB; sub++) {
                            if (sub >= nsub) break;
                            // stage and sub-step offsets added to the descriptors' address field (>> 4)
                            const uint64_t soffA = (uint64_t)((uint32_t)(stage * STAGE_A) + sub * bytesA) >> 4;
                            const uint64_t soffB = (uint64_t)((uint32_t)(stage * STAGE_B) + sub * bytesB) >> 4;
                            const uint32_t fmask = (ks == ks0 && sub == 0) ? tfresh : 0u;
#pragma unroll
                            for (int q = 0; q < MAX_MMA; q++)
                                if (q < nmma) umma(tcol[q], tad[q] + soffA, tbd[q] + soffB, tid[q], ((fmask >> q) & 1u) ^ 1u);
                        }
                        umma_commit(empty0 + 8 * stage);
                        if (++stage == NSTAGE) { stage = 0; phase ^= 1; }
                    }
                    if (!ok) break;
                    umma_commit(tfull);
                    chunk_ctr++;
                }
            }
            // all issued MMAs complete before TMEM is released
            umma_commit(finalb);
            mbar_wait(finalb, 0, status, 16u, wl);
        }
    } else {
        // ------------------------------------------------ epilogue (8 warps)
        const int quarter = warp & 3;          // TMEM lanes 32*quarter..
        const int colhalf = (warp - 2) >> 2;   // columns 32*colhalf.. of each region
        uint32_t chunk_ctr = 0;
        bool ok = true;
        for (int64_t tile = blockIdx.x; tile < total && ok; tile += gridDim.x) {
            int leafi = (int)(tile / tiles_per_leaf);
            int64_t rem = tile % tiles_per_leaf;
            int mt = (int)(rem / g.ntiles), nt = (int)(rem % g.ntiles);
            long long hi[32], lo[32];
#pragma unroll
            for (int c = 0; c < 32; c++) hi[c] = lo[c] = 0;
            for (int ch = 0; ch < nchunks; ch++) {
                // warp-uniform: tcgen05.ld below is .sync.aligned
                bool got = mbar_wait(tfull, chunk_ctr & 1, status, 32u, wl);
                if (!__all_sync(0xffffffffu, got)) { ok = false; break; }
                tc_fence_after();
                for (int r = 0; r < nd; r++) {
                    uint32_t v[32];
                    uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(TN * r + 32 * colhalf);
                    tmem_ld32(taddr, v);
                    const int t = r + 2;
                    if (t <= 5) {
                        const int sh = 7 * (5 - t);
#pragma unroll
                        for (int c = 0; c < 32; c++)
                            hi[c] += (long long)__float2int_rn(__uint_as_float(v[c])) << sh;
                    } else {
                        const int sh = 7 * (9 - t);
#pragma unroll
                        for (int c = 0; c < 32; c++)
                            lo[c] += (long long)__float2int_rn(__uint_as_float(v[c])) << sh;
                    }
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(tempty);
                chunk_ctr++;
            }
            if (!ok) break;
            // C = (hi 2^28 + lo) 2^(49 - f_i - g_j), one rounding
            const char *leaf = leaf_scalars(ws, g, leafi);
            const int64_t M = g.m;
            int64_t i = (int64_t)mt * TM + quarter * 32 + lane;
            if (i < M) {
                int fa = reinterpret_cast<const int *>(leaf + g.off_fa)[i];
                const int *fbp = reinterpret_cast<const int *>(leaf + g.off_fb);
                double *C = tasks[leafi].C;
#pragma unroll
                for (int c = 0; c < 32; c++) {
                    int64_t j = (int64_t)nt * TN + 32 * colhalf + c;
                    if (j < M) {
                        double v = fma((double)hi[c], 268435456.0, (double)lo[c]);
                        C[i + j * M] = ldexp(v, 49 - fa - fbp[j]);
                    }
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
    }
}

static int g_num_sms = 0;
static cudaError_t g_prepare_error = cudaSuccess;
static int g_prepared_device = -1;

// Sets the GEMM kernel's shared-memory attribute once per device (also
// called before a stream capture, where attribute calls are better avoided).
void split_gemm_prepare() {
    int dev = 0;
    cudaGetDevice(&dev);
    if (g_prepared_device == dev) return;
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sms <= 0) g_num_sms = 152;
    const size_t smem = (size_t)NSTAGE * STAGE_BYTES + 1024 + 1024;
    g_prepare_error = cudaFuncSetAttribute(split_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (g_prepare_error == cudaSuccess) g_prepare_error = crt_prepare();
    g_prepared_device = dev;
}

cudaError_t launch_split_scan(const LeafTask *tasks_dev, int count, int m, SplitParams p, void *workspace,
                              cudaStream_t stream) {
    Geo g = make_geo(m, count, p.scheme);
    cudaError_t e = cudaMemsetAsync(workspace, 0, g.dg_base, stream);
    if (e != cudaSuccess) return e;
    const int64_t M = m;
    const int64_t aunits = ((M + SCAN_AROWS - 1) / SCAN_AROWS) * ((M + SCAN_KSLAB - 1) / SCAN_KSLAB);
    const int64_t bunits = (M + SCAN_BCOLS - 1) / SCAN_BCOLS;
    const int64_t items = (aunits > bunits ? aunits : bunits) * count;
    dim3 grid((unsigned)(items < 4096 ? items : 4096), 2);
    split_scan_kernel<<<grid, 256, 0, stream>>>(tasks_dev, (char *)workspace, g);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_split_prep(const LeafTask *tasks_dev, int count, int m, SplitParams p, void *workspace,
                              cudaStream_t stream) {
    Geo g = make_geo(m, count, p.scheme);
    char *ws = (char *)workspace;
    {
        dim3 grid((unsigned)((m + 255) / 256), (unsigned)count);
        split_finalize_kernel<<<grid, 256, 0, stream>>>(ws, g);
        count_launch();
    }
    // the scheme, written into the header; of the two slicers below, the one
    // for the other scheme returns at once
    cudaError_t e = launch_crt_resolve(count, m, p, ws, stream);
    if (e != cudaSuccess) return e;
    e = launch_crt_slice(tasks_dev, count, m, p, ws, stream);
    if (e != cudaSuccess) return e;
    // a forced residue scheme always runs when the leaves fit it (L <= 17 for
    // 55-bit operands and K <= 2048): the digit kernels need no launch
    if (p.scheme == SCHEME_RESIDUES && g.residues_ok) return cudaSuccess;
    {
        int64_t atiles = (int64_t)g.mtiles * g.nks;
        int64_t btiles2 = ((int64_t)g.ntiles * g.nks + 1) / 2;
        int64_t items = (atiles > btiles2 ? atiles : btiles2) * count;
        dim3 grid((unsigned)(items < 4096 ? items : 4096), 2);
        split_slice_kernel<<<grid, 256, 0, stream>>>(tasks_dev, m, ws, g, p);
        count_launch();
    }
    return cudaGetLastError();
}

static int g_debug_starve = 0;
void set_debug_starve(int count) { g_debug_starve = count > 0 ? count : 0; }

cudaError_t launch_split_gemm(const LeafTask *tasks_dev, int count, int m, SplitParams p, void *workspace,
                              unsigned int *status_dev, cudaStream_t stream) {
    // one starved call covers both GEMM launches (the one for the scheme not
    // chosen returns at once)
    const int starve = g_debug_starve > 0 ? 1 : 0;
    if (starve) g_debug_starve--;
    Geo g = make_geo(m, count, p.scheme);
    char *ws = (char *)workspace;
    cudaError_t e;
    split_gemm_prepare();
    const size_t smem = (size_t)NSTAGE * STAGE_BYTES + 1024 + 1024;
    e = g_prepare_error;
    if (e != cudaSuccess) return e;
    if (!(p.scheme == SCHEME_RESIDUES && g.residues_ok)) {  // see launch_split_prep
        int64_t total = (int64_t)g.mtiles * g.ntiles * count;
        int grid = (int)(total < g_num_sms ? total : g_num_sms);
        split_gemm_kernel<<<grid, GEMM_THREADS, smem, stream>>>(tasks_dev, count, ws, g, p, status_dev, starve);
        count_launch();
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return launch_crt_gemm(tasks_dev, count, m, p, ws, status_dev, g_num_sms, stream, starve);
}

}  // namespace caps
