// Residue scheme of the split base case (Ozaki scheme II: an integer modular
// technique), on tcgen05 tensor cores.
//
// The reference multiplies leaves with FP64 dgemm (multiply.cpp:1124,
// dgemm-blas.cpp:4-13).  This scheme computes the same leaf product
// C = A * B (column-major m x m, m <= 2048) as follows:
//
//  1. scale (shared with the digit scheme): per row i of A the exponent
//     bound E_i and lowest set bit, per column j of B the same; t_a, t_b =
//     min(bits needed over the launch group, 55, the cap SplitParams.bits);
//     A'_ik = round(a_ik 2^(t_a - E_i)), B'_kj = round(b_kj 2^(t_b - E_j)),
//     |A'| <= 2^t_a, |B'| <= 2^t_b, exact when the data needs <= t bits.
//  2. resolve: the fewest moduli L whose product M_L exceeds
//     2 * K * 2^(t_a + t_b) (so C' = A'B' is fixed by its residues), and the
//     scheme: residues wherever they fit (K <= 2048), digits otherwise.
//  3. slice:   residues of A', B' modulo the pairwise coprime moduli
//     p_l in {181, 180, 179, 173, ...} (balanced, |r| <= 90, exact in bf16),
//     written as pre-tiled UMMA canonical K-major planes like the digits.
//  4. gemm:    per modulus, sum_k rA rB on tcgen05.mma kind::f16
//     (bf16 x bf16 -> f32): |sum| <= K 90^2 < 2^24 for K <= 2048, so the
//     fp32 accumulator is exact.  A's residues are premultiplied by
//     y_l = (M_L / p_l)^-1 mod p_l, so the sum is y_l A'B' mod p_l; drain
//     warps reduce it to z_l in [0, p_l), one byte per element, in a
//     product-residue tile of the CTA.
//  5. CRT (reconstruction warps of the same kernel, overlapping the next
//     tile's MMAs): S = sum_l z_l (M_L / p_l) < L M_L is reduced modulo M_L
//     and centred into (-M_L/2, M_L/2): that is C' exactly; then
//     C = C' 2^(E_i + E_j - t_a - t_b) with one rounding to FP64.
//
// Against the digit scheme's 36 digit-pair products for float data, this
// takes 17 modular products for the same 55-bit operand truncation, and its
// product of the truncated operands is exact (no dropped digit pairs).
#include "split_common.cuh"

namespace caps {

using namespace split;

namespace {

// moduli, largest first; any prefix is pairwise coprime
constexpr int MODULI[LMAX] = {181, 180, 179, 173, 169, 167, 163, 161, 157,
                              151, 149, 139, 137, 131, 127, 121, 113};

constexpr int RSTAGE_K = 4;                       // 16-deep K steps per stage (K = 64)
constexpr int RNSTAGE = 4;
constexpr int RA_TILE = TM * TK * 2;              // 4 KiB: 128 x 16 bf16
constexpr int RB_TILE = RTN * TK * 2;             // 8 KiB: 256 x 16 bf16
constexpr int RSTAGE_A = RSTAGE_K * RA_TILE;      // 16 KiB
constexpr int RSTAGE_B = RSTAGE_K * RB_TILE;      // 32 KiB
constexpr int RSTAGE_BYTES = RSTAGE_A + RSTAGE_B; // 48 KiB
constexpr int RGEMM_THREADS = 448;                // producer, MMA, 8 drain, 4 reconstruction warps
constexpr unsigned RSTATUS = 0x100;               // status bits of this kernel: RSTATUS << code

struct CrtTables {
    // the slicer's constants, each in both lanes of a float2 for the packed
    // fp32 pair instructions: -p_l, 1/p_l, c and cy below
    float2 np2[LMAX], invp2[LMAX];
    float2 c2[LMAX][3];
    float2 cy2[LMAX][LMAX][4];
    float p[LMAX], invp[LMAX];
    float c[LMAX][3];              // balanced 2^(14k) mod p_l, k = 1..3
    float cy[LMAX][LMAX][4];       // [L-1][l][k]: balanced 2^(14k) y_l mod p_l, k = 0..3,
                                   // y_l = (M_L / p_l)^-1 mod p_l
    int lg[LMAX + 1];              // lg[L] = floor(log2 M_L)
    uint32_t Ml[LMAX][LMAX][4];    // [L-1][l]: limbs of M_L / p_l, least significant first
    uint32_t M[LMAX][4];           // [L-1]: limbs of M_L
    float m_inv[LMAX];             // [L-1]: 1 / M_L
};

__constant__ CrtTables c_crt;

typedef unsigned __int128 u128;

int mod_inverse(int a, int p) {
    a %= p;
    for (int x = 1; x < p; x++)
        if ((a * x) % p == 1) return x;
    return 0;
}

void build_tables(CrtTables &t) {
    for (int l = 0; l < LMAX; l++) {
        const int p = MODULI[l];
        t.p[l] = (float)p;
        t.invp[l] = 1.0f / (float)p;
        long long v = 1;
        for (int k = 1; k <= 3; k++) {
            v = (v * 16384) % p;
            long long b = v > p / 2 ? v - p : v;
            t.c[l][k - 1] = (float)b;
            t.c2[l][k - 1] = make_float2((float)b, (float)b);
        }
        t.np2[l] = make_float2(-(float)p, -(float)p);
        t.invp2[l] = make_float2(t.invp[l], t.invp[l]);
    }
    t.lg[0] = 0;
    for (int L = 1; L <= LMAX; L++) {
        u128 M = 1;
        for (int l = 0; l < L; l++) M *= (u128)MODULI[l];
        int lg = 0;
        while ((M >> (lg + 1)) != 0) lg++;
        t.lg[L] = lg;
        for (int k = 0; k < 4; k++) t.M[L - 1][k] = (uint32_t)(M >> (32 * k));
        t.m_inv[L - 1] = (float)(1.0 / (double)M);
        for (int l = 0; l < LMAX; l++) {
            if (l >= L) {
                for (int k = 0; k < 4; k++) {
                    t.Ml[L - 1][l][k] = 0;
                    t.cy[L - 1][l][k] = 0;
                    t.cy2[L - 1][l][k] = make_float2(0.f, 0.f);
                }
                continue;
            }
            const u128 Ml = M / (u128)MODULI[l];
            const int p = MODULI[l], y = mod_inverse((int)(Ml % (u128)p), p);
            long long v = y;
            for (int k = 0; k < 4; k++) {
                t.cy[L - 1][l][k] = (float)(v > p / 2 ? v - p : v);
                t.cy2[L - 1][l][k] = make_float2(t.cy[L - 1][l][k], t.cy[L - 1][l][k]);
                v = (v * 16384) % p;
            }
            for (int k = 0; k < 4; k++) t.Ml[L - 1][l][k] = (uint32_t)(Ml >> (32 * k));
        }
    }
}


// 1.5 * 2^23: adding it to a float of magnitude below 2^22 rounds that float
// to an integer (one rounding of the exact sum), and the low bits of the
// sum's encoding then hold the integer.  Keeps rounding and int <-> float
// conversion on the FMA pipe instead of the conversion unit.
constexpr float MAGIC = 12582912.0f;

__device__ __forceinline__ float small_int_to_float(int a) {  // |a| < 2^22
    return __int_as_float(0x4B400000 + a) - MAGIC;
}

// Residues of X = round(x 2^f) modulo the first L moduli, balanced
// (|r| <= 90).  X (|X| <= 2^55) is cut into four balanced 14-bit limbs a_k
// (X + 8192 (1 + 2^14 + 2^28 + 2^42) has ordinary base-16384 digits
// a_k + 8192; |a_k| <= 8192); then y = sum_k a_k (2^(14k) mod p), balanced,
// has |y| < 2^21.1 and is exact in fp32, and r = y - p q with q = y * fl(1/p)
// rounded to an integer by one fused multiply-add with MAGIC.  That product
// is within |y / p| 2^-24 <= 2^-9.7 of y / p, while y / p lies at least
// 1/(2p) >= 2^-8.5 from a half-integer (or exactly on one for p = 180, where
// either neighbour gives |r| = 90), so q is a nearest integer and |r| <= p/2.
struct Limbs {
    float a[4];
};

// The limbs of X = round(x 2^f) (ties to even; scaled_round in
// split_common.cuh computes the same X), on 32-bit operations: from the two
// halves of x's encoding (M 2^e, M below 2^53), q = M shifted by e + f, then
// the base-16384 digits of X + 8192 (1 + 2^14 + 2^28 + 2^42) less 8192.  For
// the slicer's f (t - E with E the row's exponent bound, t <= 55) the shift
// e + f is at most 3.  Rounding right by r: q = M >> r, plus one when the bit
// below q is set and a lower bit is set or q is odd.  Checked equal to the
// 64-bit formulation on 40 million doubles and shifts, ties, subnormals and
// zeros included; it takes fewer integer instructions.
__device__ __forceinline__ Limbs scaled_limbs14(double x, int f) {
    const uint32_t hi = (uint32_t)__double2hiint(x), lo = (uint32_t)__double2loint(x);
    const int field = (int)((hi >> 20) & 0x7FFu);
    const uint32_t mh = (hi & 0xFFFFFu) | (field ? 0x100000u : 0u);
    const int sh = (field ? field - 1075 : -1074) + f;
    uint32_t ql, qh;
    if (sh >= 0) {  // at most 3
        ql = lo << sh;
        qh = __funnelshift_l(lo, mh, sh);
    } else if (sh >= -53) {
        const int r1 = -sh - 1;  // 0..52: M >> r1 ends in the round bit
        uint32_t tl, th;
        bool sticky;             // any bit below the round bit
        if (r1 < 32) {
            tl = __funnelshift_r(lo, mh, r1);
            th = mh >> r1;
            sticky = ((lo << (31 - r1)) << 1) != 0u;
        } else {
            tl = mh >> (r1 - 32);
            th = 0u;
            sticky = lo != 0u || ((mh << (63 - r1)) << 1) != 0u;
        }
        ql = __funnelshift_r(tl, th, 1);
        qh = th >> 1;
        const uint32_t up = tl & ((sticky ? 1u : 0u) | ql) & 1u;
        ql += up;
        qh += ql < up ? 1u : 0u;
    } else {        // |x 2^f| < 1/2
        ql = qh = 0u;
    }
    const uint64_t q = ((uint64_t)qh << 32) | ql;
    const uint64_t OFF = 0x0080020008002000ull;  // 8192 * sum_{k<4} 16384^k
    const uint64_t U = (hi >> 31) ? OFF - q : OFF + q;
    const uint32_t ul = (uint32_t)U, uh = (uint32_t)(U >> 32);
    Limbs l;
    l.a[0] = small_int_to_float((int)(ul & 16383u) - 8192);
    l.a[1] = small_int_to_float((int)((ul >> 14) & 16383u) - 8192);
    l.a[2] = small_int_to_float((int)(__funnelshift_r(ul, uh, 28) & 16383u) - 8192);
    l.a[3] = small_int_to_float((int)(uh >> 10) - 8192);
    return l;
}

// The balanced residues (|r| <= 90) of two values' integers modulo p_l, one
// per lane, on packed fp32 pair instructions: each lane performs exactly
// the scalar sequence y = a0 + a1 c0 + a2 c1 + a3 c2 (three fused
// multiply-adds, innermost first), q = fl(y fl(1/p) + MAGIC) - MAGIC,
// r = fl(y - q p), with round-to-nearest per lane as the scalar forms, at
// half the issued instructions.
struct Limbs2 {
    float2 a[4];  // lane x: the first value's limbs, lane y: the second's
};

__device__ __forceinline__ Limbs2 pair_limbs(const Limbs &u, const Limbs &v) {
    Limbs2 x;
#pragma unroll
    for (int k = 0; k < 4; k++) x.a[k] = make_float2(u.a[k], v.a[k]);
    return x;
}

__device__ __forceinline__ float2 reduce_pair(float2 y, int l) {
    const float2 q = __fadd2_rn(__ffma2_rn(y, c_crt.invp2[l], make_float2(MAGIC, MAGIC)),
                                make_float2(-MAGIC, -MAGIC));
    return __ffma2_rn(q, c_crt.np2[l], y);
}

__device__ __forceinline__ float2 residue_pair(const Limbs2 &x, int l) {
    const float2 *c = c_crt.c2[l];
    return reduce_pair(__ffma2_rn(x.a[3], c[2], __ffma2_rn(x.a[2], c[1], __ffma2_rn(x.a[1], c[0], x.a[0]))), l);
}

// the same for the integers times y_l (the CRT coefficient of modulus l among
// L): A's residues carry y_l, so each modulus's product sum is already
// y_l A'B' mod p_l, the term the CRT needs.  |y| <= 4 * 8192 * 90 < 2^21.5,
// so y / p is within 2^-9.3 of y * fl(1/p), still inside the half-integer
// margin of 2^-8.5.
__device__ __forceinline__ float2 residue_y_pair(const Limbs2 &x, int L, int l) {
    const float2 *cy = c_crt.cy2[L - 1][l];
    return reduce_pair(
        __ffma2_rn(x.a[3], cy[3], __ffma2_rn(x.a[2], cy[2], __ffma2_rn(x.a[1], cy[1], __fmul2_rn(x.a[0], cy[0])))),
        l);
}

// two residues as packed bf16: |r| <= 90 has at most 7 significant bits, so
// the top half of its fp32 encoding is its exact bf16 encoding
__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    return __byte_perm(__float_as_uint(lo), __float_as_uint(hi), 0x7632);
}

}  // namespace

int crt_moduli_needed(int bits, int K) {
    const int Kp = (K + TK - 1) / TK * TK;
    int kb = 0;
    while ((1 << kb) < Kp) kb++;
    const int need = 2 * bits + kb + 1;  // as crt_resolve_kernel: K 2^(ta+tb) < M_L / 2
    u128 M = 1;
    for (int L = 1; L <= LMAX; L++) {
        M *= (u128)MODULI[L - 1];
        int lg = 0;
        while ((M >> (lg + 1)) != 0) lg++;
        if (lg >= need) return L;
    }
    return 0;
}

// ---------------------------------------------------------------- resolve
// One thread: picks the scheme for the launch group from the scan's results
// and writes it into the header, where every later kernel of the group reads it.
__global__ void crt_resolve_kernel(char *__restrict__ ws, Geo g, SplitParams p) {
    if (threadIdx.x != 0) return;
    SplitHdr *h = reinterpret_cast<SplitHdr *>(ws);
    int s, nd;
    resolve_sd(h, p, s, nd);
    h->s_used = s;
    h->nd_used = nd;
    const bool forced_digits = p.scheme == SCHEME_DIGITS || (p.scheme == SCHEME_AUTO && p.slices > 0);
    // operand bits: what the data need, at most 55, at most the cap asked for
    // (a cap only where the residues run: the digit scheme sets its own cut)
    const int cap = (p.bits > 0 && p.bits < 55 && !forced_digits) ? p.bits : 55;
    const int ta = h->bitsA < cap ? h->bitsA : cap, tb = h->bitsB < cap ? h->bitsB : cap;
    int residues = 0, L = 0;
    if (g.residues_ok && !forced_digits) {
        int kb = 0;
        while ((1 << kb) < g.Kp) kb++;
        const int need = ta + tb + kb + 1;  // K 2^(ta+tb) < M_L / 2
        L = 1;
        while (L <= LMAX && c_crt.lg[L] < need) L++;
        // wherever the residues fit they are the faster cut, integer data
        // included: the digit GEMM's per-chunk drain of its diagonal
        // accumulators costs about as much at one digit as at eight
        if (L <= LMAX) residues = 1;
    }
    h->ta = ta;
    h->tb = tb;
    h->moduli = residues ? L : 0;
    h->residues = residues;
}

// ---------------------------------------------------------------- slice
// The residues of 4 pairs of values modulo each of the first NL moduli (A
// side: premultiplied by the CRT coefficients of NL moduli), 8 bf16 per plane.
template <int NL>
__device__ __forceinline__ void write_residues_unrolled(const Limbs2 (&x)[4], char *dst, size_t plane_stride,
                                                        int side) {
    if (side == 0) {
#pragma unroll
        for (int l = 0; l < NL; l++) {
            uint32_t w[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const float2 r = residue_y_pair(x[q], NL, l);
                w[q] = pack_bf16x2(r.x, r.y);
            }
            *reinterpret_cast<uint4 *>(dst + (size_t)l * plane_stride) = make_uint4(w[0], w[1], w[2], w[3]);
        }
    } else {
#pragma unroll
        for (int l = 0; l < NL; l++) {
            uint32_t w[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const float2 r = residue_pair(x[q], l);
                w[q] = pack_bf16x2(r.x, r.y);
            }
            *reinterpret_cast<uint4 *>(dst + (size_t)l * plane_stride) = make_uint4(w[0], w[1], w[2], w[3]);
        }
    }
}

// Residue planes, per modulus l:
//   A: [l][mt][ks] tiles of 128 x 16 (4 KiB), B: [l][rt][ks] tiles of 256 x 16
//   (8 KiB), each the UMMA canonical K-major image (8-row x 16-byte core
//   matrices, K halves side by side: K stride 128 B, row-group stride 256 B).
// A side: one thread = one row x 8 k, a block = one 128 x 16 tile.  B side:
// one thread = one column x 8 k, a block = half of a 256 x 16 tile.
__device__ __forceinline__ void crt_slice_tile(const LeafTask *__restrict__ tasks, char *__restrict__ ws,
                                               const Geo &g, const SplitHdr *h, int L, int leaf, int64_t tile,
                                               int side) {
    const LeafTask t = tasks[leaf];
    const char *sc = leaf_scalars(ws, g, leaf);
    char *pl = leaf_digits(ws, g, leaf);
    const int64_t M = g.m;
    const int tid = threadIdx.x;
    const int kg = tid >> 7;  // which 8 of the tile's 16 k
    int64_t idx, k0, sk;      // row of A / column of B, first k, stride between k
    const double *src;
    int ee, tt;
    char *dst;
    size_t plane_stride;
    if (side == 0) {
        if (tile >= (int64_t)g.mtiles * g.nks) return;
        const int mt = (int)(tile / g.nks), ks = (int)(tile % g.nks);
        const int r = tid & 127;
        idx = (int64_t)mt * TM + r;
        k0 = (int64_t)ks * TK + kg * 8;
        src = t.A + idx + k0 * M;
        sk = M;
        ee = idx < M ? reinterpret_cast<const int *>(sc + g.off_ea)[idx] : 0;
        tt = h->ta;
        dst = pl + g.off_ra + ((size_t)mt * g.nks + ks) * RA_TILE + (size_t)(r >> 3) * 256 + (size_t)kg * 128 +
              (size_t)(r & 7) * 16;
        plane_stride = (size_t)g.mtiles * g.nks * RA_TILE;
    } else {
        if (tile >= (int64_t)g.rtiles * g.nks * 2) return;
        const int64_t bt = tile >> 1;
        const int rt = (int)(bt / g.nks), ks = (int)(bt % g.nks);
        const int c = (int)(tile & 1) * 128 + (tid & 127);
        idx = (int64_t)rt * RTN + c;
        k0 = (int64_t)ks * TK + kg * 8;
        src = t.B + k0 + idx * M;
        sk = 1;
        ee = idx < M ? reinterpret_cast<const int *>(sc + g.off_eb)[idx] : 0;
        tt = h->tb;
        dst = pl + g.off_rb + ((size_t)rt * g.nks + ks) * RB_TILE + (size_t)(c >> 3) * 256 + (size_t)kg * 128 +
              (size_t)(c & 7) * 16;
        plane_stride = (size_t)g.rtiles * g.nks * RB_TILE;
    }
    // f = t - E (ee = E + 4096; 0 for a zero row / column); padding rows,
    // columns and k give zero residues
    const bool live = idx < M && ee != 0;
    const int f = tt - (ee - 4096);
    double v[8];
#pragma unroll
    for (int e = 0; e < 8; e++) v[e] = (live && k0 + e < M) ? __ldg(src + e * sk) : 0.0;
    Limbs2 x[4];
#pragma unroll
    for (int q = 0; q < 4; q++) x[q] = pair_limbs(scaled_limbs14(v[2 * q], f), scaled_limbs14(v[2 * q + 1], f));
    switch (L) {
        // float data need 17 moduli at 55 bits, 16 or 15 under an operand-bit
        // cap: unrolled, the constants' addresses are fixed, with no
        // per-modulus address arithmetic or loop bookkeeping
        case 17: write_residues_unrolled<17>(x, dst, plane_stride, side); break;
        case 16: write_residues_unrolled<16>(x, dst, plane_stride, side); break;
        case 15: write_residues_unrolled<15>(x, dst, plane_stride, side); break;
        default:
#pragma unroll 1
            for (int l = 0; l < L; l++) {
                uint32_t w[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const float2 r = side == 0 ? residue_y_pair(x[q], L, l) : residue_pair(x[q], l);
                    w[q] = pack_bf16x2(r.x, r.y);
                }
                *reinterpret_cast<uint4 *>(dst + (size_t)l * plane_stride) = make_uint4(w[0], w[1], w[2], w[3]);
            }
    }
}

// Grid-stride over (leaf, tile), so that the launch is cheap when the digit
// scheme runs and this kernel returns at once.  blockIdx.y: A (0) or B (1).
__global__ void __launch_bounds__(256) crt_slice_kernel(const LeafTask *__restrict__ tasks,
                                                        char *__restrict__ ws, Geo g) {
    const SplitHdr *h = reinterpret_cast<const SplitHdr *>(ws);
    if (!h->residues) return;  // the digit scheme runs
    const int L = h->moduli;
    const int64_t atiles = (int64_t)g.mtiles * g.nks, bhalves = (int64_t)g.rtiles * g.nks * 2;
    const int64_t per = atiles > bhalves ? atiles : bhalves;
    const int64_t total = per * g.count;
    for (int64_t it = blockIdx.x; it < total; it += gridDim.x)
        crt_slice_tile(tasks, ws, g, h, L, (int)(it / per), it % per, blockIdx.y);
}

// ---------------------------------------------------------------- CRT reconstruction
namespace {

// The encoding of the double nearest |v| 2^e (ties to even), with the sign
// of v, for |v| = hi 2^64 + lo < 2^127.  One rounding: the integer is rounded
// at the result's last place -- 53 significant bits, or 2^-1074 for a
// subnormal result -- and the encoding is then assembled with integer
// operations (the FP64 pipe runs at 1/64 of FP32 here): for a significand
// m <= 2^53 whose last place is 2^ex, the bits are ((ex + 1074) << 52) + m,
// which also covers subnormals (ex = -1074, m < 2^52) and a rounding carry
// into the exponent.
__device__ __forceinline__ unsigned long long round_scaled_bits(uint64_t hi, uint64_t lo, bool neg, int e) {
    if ((hi | lo) == 0) return 0;
    const int nb = hi ? 128 - __clzll((long long)hi) : 64 - __clzll((long long)lo);
    int ex = nb - 53 + e;
    if (ex < -1074) ex = -1074;
    const int s = ex - e;  // right shift of |v| that leaves the significand
    uint64_t mant;
    if (s <= 0) {
        mant = lo << (-s);  // |v| < 2^53 here
    } else if (s >= 128) {
        mant = 0;           // below half of 2^-1074
    } else {
        uint64_t q, rb, st;
        if (s < 64) {
            q = (lo >> s) | (hi << (64 - s));
            rb = (lo >> (s - 1)) & 1;
            st = lo & ((1ull << (s - 1)) - 1);
        } else if (s == 64) {
            q = hi;
            rb = lo >> 63;
            st = lo << 1;
        } else {
            q = hi >> (s - 64);
            rb = (hi >> (s - 65)) & 1;
            st = (hi & ((1ull << (s - 65)) - 1)) | lo;
        }
        mant = q + (rb & ((st != 0) | (q & 1)));
    }
    const unsigned long long sign = neg ? 0x8000000000000000ull : 0ull;
    if (ex > 971) return sign | 0x7FF0000000000000ull;  // |result| >= 2^1024
    return sign | (((unsigned long long)(ex + 1074) << 52) + mant);
}

// The same for the common case, without divergent branches: |v| is shifted
// so that its top bit is bit 127 (top: bits 127..64, rest: 63..0); a normal
// result's significand is then top >> 11, its round bit top bit 10 and its
// sticky bits the rest.  Results below the normal range take the general path.
__device__ __forceinline__ unsigned long long round_scaled_bits_fast(uint64_t hi, uint64_t lo, bool neg, int e) {
    if ((hi | lo) == 0) return 0;
    const int lz = hi ? __clzll((long long)hi) : 64 + __clzll((long long)lo);
    const int ex = 128 - lz - 53 + e;  // last place of a normal result
    if (ex < -1074) return round_scaled_bits(hi, lo, neg, e);
    uint64_t top, rest;
    if (lz >= 64) {
        top = lo << (lz - 64);
        rest = 0;
    } else if (lz == 0) {
        top = hi;
        rest = lo;
    } else {
        top = (hi << lz) | (lo >> (64 - lz));
        rest = lo << lz;
    }
    uint64_t mant = top >> 11;
    const uint64_t rb = (top >> 10) & 1, st = (top & 0x3FFull) | rest;
    mant += rb & ((st != 0) | (mant & 1));
    const unsigned long long sign = neg ? 0x8000000000000000ull : 0ull;
    if (ex > 971) return sign | 0x7FF0000000000000ull;  // |result| >= 2^1024
    return sign | (((unsigned long long)(ex + 1074) << 52) + mant);
}

}  // namespace

namespace {

// C' for 4 consecutive rows of one column from their product-residue bytes:
// zq[l] holds z_l of the 4 rows (byte q = row q).  S = sum_l z_l M_L / p_l
// (< L M_L < 2^128) is formed in 32-bit limbs with 64-bit column sums; then
// qe = S / M_L rounded from an fp32 estimate of S (32-bit conversions: the
// 64-bit ones run on the FP64 pipe), C' = S - qe M_L in 32-bit limbs with a
// signed carry, and C' is centred into (-M_L/2, M_L/2] (qe may be one off
// when S / M_L lies near a half-integer).  out[q] = the FP64 encoding of
// C'_q 2^e[q], or 0 where zero[q].
__device__ __forceinline__ void crt_reconstruct4(const uint32_t (&zq)[LMAX], int L, const int (&e)[4],
                                                 const bool (&zero)[4], unsigned long long (&out)[4]) {
    uint64_t s[4][4];
#pragma unroll
    for (int q = 0; q < 4; q++)
#pragma unroll
        for (int k = 0; k < 4; k++) s[q][k] = 0;
#pragma unroll
    for (int l = 0; l < LMAX; l++) {
        if (l < L) {
            const uint32_t *ml = c_crt.Ml[L - 1][l];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const uint32_t z = (zq[l] >> (8 * q)) & 255u;
#pragma unroll
                for (int k = 0; k < 4; k++) s[q][k] += (uint64_t)z * ml[k];
            }
        }
    }
    uint32_t Mw[4];
#pragma unroll
    for (int k = 0; k < 4; k++) Mw[k] = c_crt.M[L - 1][k];
    const u128 Mv = ((u128)(((uint64_t)Mw[3] << 32) | Mw[2]) << 64) | (((uint64_t)Mw[1] << 32) | Mw[0]);
    const u128 Mhalf = Mv >> 1;
    const float minv = c_crt.m_inv[L - 1];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        uint32_t w[4];
        uint64_t c = s[q][0];
        w[0] = (uint32_t)c;
        c = s[q][1] + (c >> 32);
        w[1] = (uint32_t)c;
        c = s[q][2] + (c >> 32);
        w[2] = (uint32_t)c;
        c = s[q][3] + (c >> 32);
        w[3] = (uint32_t)c;
        const float sf = fmaf((float)w[3], 7.9228162514264337593543950336e28f,
                              fmaf((float)w[2], 18446744073709551616.0f, fmaf((float)w[1], 4294967296.0f, (float)w[0])));
        const long long qe = (long long)__float2int_rn(sf * minv);
        long long t = 0;
        uint32_t r[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            t += (long long)w[k] - qe * (long long)Mw[k];
            r[k] = (uint32_t)t;
            t >>= 32;
        }
        const u128 Cr = ((u128)(((uint64_t)r[3] << 32) | r[2]) << 64) | (((uint64_t)r[1] << 32) | r[0]);
        bool neg = (r[3] >> 31) != 0;
        u128 mag = neg ? (u128)0 - Cr : Cr;
        if (mag > Mhalf) {
            mag = Mv - mag;  // C' -+ M_L has the other sign
            neg = !neg;
        }
        out[q] = zero[q] ? 0ull : round_scaled_bits_fast((uint64_t)(mag >> 64), (uint64_t)mag, neg, e[q]);
    }
}

}  // namespace

// ---------------------------------------------------------------- gemm
// Persistent, one CTA per SM, 448 threads: warp 0 loads (one lane, bulk
// copies of pre-tiled planes), warp 1 issues the MMAs (one lane), warps 2..9
// drain the accumulators, warps 10..13 reconstruct C.
//
// A work unit is (leaf, 128-row tile, 256-column tile).  For each modulus in
// turn it takes Kp / 16 MMAs of 128 x 256 x 16 into one of two TMEM
// accumulators of 256 columns; they alternate, so the drain of one modulus
// overlaps the MMAs of the next.  The drain reduces each exact sum modulo p
// and stores z = (c mod p) y mod p as a byte into the CTA's product-residue
// tile: [modulus][column][row], two tiles per CTA used in turn.  When a
// unit's last modulus is drained, the four reconstruction warps turn that
// tile into C (CRT, one rounding) while the drain moves on to the next unit's
// moduli in the other tile; mbarriers hand the tiles back and forth.
//
// Units are ordered leaf, row tile, column tile, and the CTAs go through the
// moduli in step, so the CTAs running at one time share the A and B planes
// of one modulus of about one leaf (16 MB at m = 2048) through L2.
__global__ void __launch_bounds__(RGEMM_THREADS, 1)
    crt_gemm_kernel(const LeafTask *__restrict__ tasks, char *__restrict__ ws, Geo g,
                    unsigned *__restrict__ status, int starve) {
    const SplitHdr *h = reinterpret_cast<const SplitHdr *>(ws);
    if (!h->residues) return;  // the digit scheme runs
    const int L = h->moduli;
    // starve (test hook): no copies are issued, so nothing is ever in flight
    // and every wait may give up after a short spin
    const uint32_t wl = starve ? WAIT_LIMIT_STARVED : WAIT_LIMIT;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char *stA = smem;                        // RNSTAGE x RSTAGE_A
    unsigned char *stB = smem + RNSTAGE * RSTAGE_A;   // RNSTAGE x RSTAGE_B
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + RNSTAGE * RSTAGE_BYTES);
    // bars: full[RNSTAGE], empty[RNSTAGE], tfull[2], tempty[2], final, zfull[2], zempty[2]
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * RNSTAGE + 9);
    const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + RNSTAGE);
    const uint32_t tfull0 = smem_u32(bars + 2 * RNSTAGE), tempty0 = smem_u32(bars + 2 * RNSTAGE + 2);
    const uint32_t finalb = smem_u32(bars + 2 * RNSTAGE + 4);
    const uint32_t zfull0 = smem_u32(bars + 2 * RNSTAGE + 5), zempty0 = smem_u32(bars + 2 * RNSTAGE + 7);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        for (int i = 0; i < RNSTAGE; i++) {
            mbar_init(full0 + 8 * i, 1);
            mbar_init(empty0 + 8 * i, 1);
        }
        for (int i = 0; i < 2; i++) {
            mbar_init(tfull0 + 8 * i, 1);
            mbar_init(tempty0 + 8 * i, 8);   // the 8 drain warps
            mbar_init(zfull0 + 8 * i, 8);    // the 8 drain warps
            mbar_init(zempty0 + 8 * i, 4);   // the 4 reconstruction warps
        }
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

    const int64_t tiles = (int64_t)g.mtiles * g.rtiles;
    const int64_t total = tiles * g.count;
    const int nks = g.nks;
    unsigned char *ztiles = (unsigned char *)ws + g.z_base + (size_t)blockIdx.x * 2 * ZTILE_BYTES;

    if (warp == 0) {
        // ------------------------------------------------ producer
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            bool ok = true;
            uint32_t armed[RNSTAGE] = {0, 0, 0, 0};  // 1 + phase of the last arm
            for (int64_t u = blockIdx.x; u < total && ok && !starve; u += gridDim.x) {
                const int leafi = (int)(u / tiles);
                const int64_t tile = u % tiles;
                const int mt = (int)(tile / g.rtiles), rt = (int)(tile % g.rtiles);
                const char *pl = leaf_digits(ws, g, leafi);
                for (int l = 0; l < L && ok; l++) {
                    const char *srcA = pl + g.off_ra + (((size_t)l * g.mtiles + mt) * nks) * RA_TILE;
                    const char *srcB = pl + g.off_rb + (((size_t)l * g.rtiles + rt) * nks) * RB_TILE;
                    for (int ks = 0; ks < nks; ks += RSTAGE_K) {
                        const uint32_t n = ks + RSTAGE_K <= nks ? RSTAGE_K : (uint32_t)(nks - ks);
                        if (!mbar_wait(empty0 + 8 * stage, phase ^ 1, status, RSTATUS << 0, wl)) { ok = false; break; }
                        mbar_expect_tx(full0 + 8 * stage, n * (RA_TILE + RB_TILE));
                        bulk_g2s(smem_u32(stA + stage * RSTAGE_A), srcA + (size_t)ks * RA_TILE, n * RA_TILE,
                                 full0 + 8 * stage);
                        bulk_g2s(smem_u32(stB + stage * RSTAGE_B), srcB + (size_t)ks * RB_TILE, n * RB_TILE,
                                 full0 + 8 * stage);
                        armed[stage] = 1 + phase;
                        if (++stage == RNSTAGE) { stage = 0; phase ^= 1; }
                    }
                }
            }
            // every armed stage's copies land before the CTA exits
            for (int i = 0; i < RNSTAGE; i++)
                if (armed[i]) mbar_wait(full0 + 8 * i, armed[i] - 1, status, RSTATUS << 1, wl);
        }
    } else if (warp == 1) {
        // ------------------------------------------------ MMA issuer
        if (lane == 0) {
            // K-direction core-matrix stride (LBO) 128 B, row-group stride (SBO) 256 B
            const uint64_t a0 = sdesc(smem_u32(stA), 128, 256), b0 = sdesc(smem_u32(stB), 128, 256);
            const uint32_t idesc = idesc_bf16(TM, RTN);
            int stage = 0;
            uint32_t phase = 0, uc = 0;
            bool ok = true;
            for (int64_t u = blockIdx.x; u < total && ok; u += gridDim.x) {
                for (int l = 0; l < L && ok; l++, uc++) {
                    const uint32_t acc = uc & 1;
                    if (!mbar_wait(tempty0 + 8 * acc, ((uc >> 1) & 1) ^ 1, status, RSTATUS << 2, wl)) { ok = false; break; }
                    tc_fence_after();
                    const uint32_t dt = tmem + acc * RTN;
                    for (int ks = 0; ks < nks; ks += RSTAGE_K) {
                        const int n = ks + RSTAGE_K <= nks ? RSTAGE_K : nks - ks;
                        if (!mbar_wait(full0 + 8 * stage, phase, status, RSTATUS << 3, wl)) { ok = false; break; }
                        tc_fence_after();
                        const uint64_t sa = (uint64_t)((uint32_t)stage * RSTAGE_A) >> 4;
                        const uint64_t sb = (uint64_t)((uint32_t)stage * RSTAGE_B) >> 4;
#pragma unroll
                        for (int j = 0; j < RSTAGE_K; j++)
                            if (j < n)
                                umma(dt, a0 + sa + (uint64_t)(j * RA_TILE >> 4), b0 + sb + (uint64_t)(j * RB_TILE >> 4),
                                     idesc, (ks + j) > 0 ? 1u : 0u);
                        umma_commit(empty0 + 8 * stage);
                        if (++stage == RNSTAGE) { stage = 0; phase ^= 1; }
                    }
                    if (!ok) break;
                    umma_commit(tfull0 + 8 * acc);
                }
            }
            // every issued MMA completes before TMEM is released
            umma_commit(finalb);
            mbar_wait(finalb, 0, status, RSTATUS << 4, wl);
        }
    } else if (warp < 10) {
        // ------------------------------------------------ drain (8 warps)
        const int quarter = warp & 3;          // TMEM lanes 32*quarter.. (rows of the tile)
        const int colhalf = (warp - 2) >> 2;   // columns 128*colhalf.. of the tile
        const int row = quarter * 32 + lane;
        uint32_t uc = 0, tc = 0;
        bool ok = true;
        for (int64_t u = blockIdx.x; u < total && ok; u += gridDim.x, tc++) {
            const uint32_t zb = tc & 1;
            // the reconstruction warps are done with this residue tile
            const bool free_ = mbar_wait(zempty0 + 8 * zb, ((tc >> 1) & 1) ^ 1, status, RSTATUS << 6, wl);
            if (!__all_sync(0xffffffffu, free_)) break;
            unsigned char *zt = ztiles + (size_t)zb * ZTILE_BYTES + row;
            for (int l = 0; l < L; l++, uc++) {
                const uint32_t acc = uc & 1;
                // warp-uniform: tcgen05.ld below is .sync.aligned
                const bool got = mbar_wait(tfull0 + 8 * acc, (uc >> 1) & 1, status, RSTATUS << 5, wl);
                if (!__all_sync(0xffffffffu, got)) { ok = false; break; }
                tc_fence_after();
                const float p = c_crt.p[l], invp = c_crt.invp[l];
                unsigned char *out = zt + (size_t)l * RTN * TM;
#pragma unroll 1
                for (int c4 = 0; c4 < 4; c4++) {
                    uint32_t v[32];
                    const int col0 = colhalf * 128 + c4 * 32;
                    tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + acc * RTN + col0, v);
#pragma unroll
                    for (int e = 0; e < 32; e++) {
                        // c = sum rA rB = y A'B' mod p (exact, |c| < 2^24; A's
                        // residues carry y).  q = c / p rounded by MAGIC is floor
                        // or ceil of c / p (|c / p| 2^-24 < 1/2 away), so c - q p
                        // lies in [-p, p) and one correction gives z = c mod p.
                        const float c = __uint_as_float(v[e]);
                        float z = fmaf(-(fmaf(c, invp, MAGIC) - MAGIC), p, c);
                        z = z < 0.0f ? z + p : z;
                        out[(size_t)(col0 + e) * TM] = (unsigned char)__float_as_uint(z + MAGIC);  // low byte: z
                    }
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(tempty0 + 8 * acc);
            }
            if (!ok) break;
            // the tile's residues are complete: hand it to the reconstruction warps
            __threadfence_block();
            __syncwarp();
            if (lane == 0) mbar_arrive(zfull0 + 8 * zb);
        }
    } else {
        // ------------------------------------------------ reconstruction (4 warps)
        // one warp = one column of the tile at a time, each lane 4 of its rows
        const int w = warp - 10;
        const int64_t M = g.m;
        uint32_t tc = 0;
        for (int64_t u = blockIdx.x; u < total; u += gridDim.x, tc++) {
            const uint32_t zb = tc & 1;
            const bool got = mbar_wait(zfull0 + 8 * zb, (tc >> 1) & 1, status, RSTATUS << 7, wl);
            if (!__all_sync(0xffffffffu, got)) break;
            const int leafi = (int)(u / tiles);
            const int64_t tile = u % tiles;
            const int mt = (int)(tile / g.rtiles), rt = (int)(tile % g.rtiles);
            const char *sc = leaf_scalars(ws, g, leafi);
            const int *eap = reinterpret_cast<const int *>(sc + g.off_ea);
            const int *ebp = reinterpret_cast<const int *>(sc + g.off_eb);
            double *C = tasks[leafi].C;
            const int64_t i0 = (int64_t)mt * TM + lane * 4;
            int ei[4];
#pragma unroll
            for (int q = 0; q < 4; q++) ei[q] = i0 + q < M ? eap[i0 + q] : 0;
            const unsigned char *zt = ztiles + (size_t)zb * ZTILE_BYTES + lane * 4;
            // the residue words of column col; the next column's are loaded
            // before this one is reconstructed (the tiles mostly come from
            // DRAM: two per CTA exceed L2)
            uint32_t zq[LMAX], zn[LMAX];
#pragma unroll
            for (int l = 0; l < LMAX; l++)
                zq[l] = l < L ? *reinterpret_cast<const uint32_t *>(zt + ((size_t)l * RTN + w) * TM) : 0u;
#pragma unroll 1
            for (int col = w; col < RTN; col += 4) {
                const int next = col + 4 < RTN ? col + 4 : col;
#pragma unroll
                for (int l = 0; l < LMAX; l++)
                    zn[l] = l < L ? *reinterpret_cast<const uint32_t *>(zt + ((size_t)l * RTN + next) * TM) : 0u;
                const int64_t j = (int64_t)rt * RTN + col;
                if (j >= M || i0 >= M) {
#pragma unroll
                    for (int l = 0; l < LMAX; l++) zq[l] = zn[l];
                    continue;
                }
                const int ej = ebp[j];
                int e[4];
                bool zero[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    // C = C' 2^(E_i + E_j - ta - tb); a zero row / column has C' = 0
                    zero[q] = ei[q] == 0 || ej == 0;
                    e[q] = (ei[q] - 4096) + (ej - 4096) - h->ta - h->tb;
                }
                unsigned long long out[4];
                crt_reconstruct4(zq, L, e, zero, out);
                double *dst = C + i0 + j * M;
                if (i0 + 3 < M && ((uintptr_t)dst & 15) == 0) {
                    reinterpret_cast<double2 *>(dst)[0] =
                        make_double2(__longlong_as_double((long long)out[0]), __longlong_as_double((long long)out[1]));
                    reinterpret_cast<double2 *>(dst)[1] =
                        make_double2(__longlong_as_double((long long)out[2]), __longlong_as_double((long long)out[3]));
                } else {
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        if (i0 + q < M) dst[q] = __longlong_as_double((long long)out[q]);
                }
#pragma unroll
                for (int l = 0; l < LMAX; l++) zq[l] = zn[l];
            }
            // this residue tile may be refilled
            __syncwarp();
            if (lane == 0) mbar_arrive(zempty0 + 8 * zb);
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
    }
}

// ---------------------------------------------------------------- launchers
static CrtTables g_tables_host;
static bool g_tables_built = false;
static int g_crt_device = -1;
static cudaError_t g_crt_error = cudaSuccess;

cudaError_t crt_prepare() {
    int dev = 0;
    cudaGetDevice(&dev);
    if (g_crt_device == dev) return g_crt_error;
    if (!g_tables_built) {
        build_tables(g_tables_host);
        g_tables_built = true;
    }
    g_crt_error = cudaMemcpyToSymbol(c_crt, &g_tables_host, sizeof(CrtTables));
    if (g_crt_error == cudaSuccess) {
        const size_t smem = (size_t)RNSTAGE * RSTAGE_BYTES + 1024 + 1024;
        g_crt_error = cudaFuncSetAttribute(crt_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    }
    g_crt_device = dev;
    return g_crt_error;
}

cudaError_t launch_crt_resolve(int count, int m, SplitParams p, void *workspace, cudaStream_t stream) {
    // the resolve reads the moduli tables: they must be on the device before
    // the first launch group of the process (returns at once afterwards)
    cudaError_t e = crt_prepare();
    if (e != cudaSuccess) return e;
    Geo g = make_geo(m, count, p.scheme);
    crt_resolve_kernel<<<1, 32, 0, stream>>>((char *)workspace, g, p);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_crt_slice(const LeafTask *tasks_dev, int count, int m, SplitParams p, void *workspace,
                             cudaStream_t stream) {
    Geo g = make_geo(m, count, p.scheme);
    if (!g.residues_ok) return cudaSuccess;
    const int64_t atiles = (int64_t)g.mtiles * g.nks, bhalves = (int64_t)g.rtiles * g.nks * 2;
    const int64_t items = (atiles > bhalves ? atiles : bhalves) * count;
    dim3 grid((unsigned)(items < 4096 ? items : 4096), 2);
    crt_slice_kernel<<<grid, 256, 0, stream>>>(tasks_dev, (char *)workspace, g);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_crt_gemm(const LeafTask *tasks_dev, int count, int m, SplitParams p, void *workspace,
                            unsigned int *status_dev, int num_sms, cudaStream_t stream, int starve) {
    Geo g = make_geo(m, count, p.scheme);
    if (!g.residues_ok) return cudaSuccess;
    cudaError_t e = crt_prepare();
    if (e != cudaSuccess) return e;
    const int64_t units = (int64_t)g.mtiles * g.rtiles * count;
    int grid = (int)(units < num_sms ? units : num_sms);
    if (grid > ZCTA_MAX) grid = ZCTA_MAX;  // two product-residue tiles per CTA
    const size_t smem = (size_t)RNSTAGE * RSTAGE_BYTES + 1024 + 1024;
    crt_gemm_kernel<<<grid, RGEMM_THREADS, smem, stream>>>(tasks_dev, (char *)workspace, g, status_dev, starve);
    count_launch();
    return cudaGetLastError();
}

}  // namespace caps
