// Internals shared by the two split-form schemes (digit slices in
// kernels_split.cu, residue slices in kernels_crt.cu): the launch group's
// workspace layout and header, the exponent helpers and the rounding of
// x * 2^f to an integer, and the mbarrier / bulk-copy / tcgen05 wrappers.
#pragma once
#include "common.cuh"

namespace caps {
namespace split {

constexpr int TM = 128;        // rows of A per tile (TMEM lanes), both schemes
constexpr int TN = 64;         // digit scheme: columns of B per diagonal region
constexpr int TK = 16;         // K per MMA
constexpr int MAXS = 8;        // digit scheme: max digits
constexpr int RTN = 256;       // residue scheme: columns of B per tile (one MMA)
constexpr int LMAX = 17;       // residue scheme: max moduli
constexpr int RKMAX = 2048;    // residue scheme: max K (K * 90^2 < 2^24: exact fp32 sums)
constexpr int ZCTA_MAX = 160;  // residue scheme: GEMM CTAs with product-residue scratch
constexpr size_t ZTILE_BYTES = (size_t)LMAX * TM * RTN;  // product residues of one tile
constexpr uint32_t WAIT_LIMIT = 1u << 25;
// wait limit of a GEMM launch the starvation test hook runs: it issues no
// copies, so its waits have nothing in flight and may give up early
constexpr uint32_t WAIT_LIMIT_STARVED = 1u << 12;

enum { SCHEME_AUTO = 0, SCHEME_DIGITS = 1, SCHEME_RESIDUES = 2 };

// First 256 bytes of a launch group's workspace.  The host reads the first
// four fields back after a multiply (counters).
struct SplitHdr {
    int needed;    // digits needed, max over the group (finalize)
    int s_used;    // digit scheme: digits and diagonals (resolve)
    int nd_used;
    int moduli;    // residue scheme: moduli used; 0 when the digit scheme runs (resolve)
    int bitsA;     // max over rows of A of E - lsb + 1 (finalize)
    int bitsB;     // the same over the columns of B
    int residues;  // 1: the residue scheme runs (resolve)
    int ta, tb;    // residue scheme: |A'| <= 2^ta, |B'| <= 2^tb
    int pad[55];
};
static_assert(sizeof(SplitHdr) == 256, "split header is 256 bytes");

// Workspace of one launch group of `count` leaves:
//   [header 256 B][scalars of leaf 0..count-1][plane block of leaf 0..count-1]
//   [residue scheme: product-residue scratch, two tiles per GEMM CTA]
// scalars per leaf: f (A rows), g (B columns) of the digit scheme, and the
// scan's exponent / lsb encodings.  A leaf's plane block holds either the
// digit planes (A then B, pre-tiled) or, for the residue scheme, the residue
// planes of A and B; it is sized for the larger.
struct Geo {
    int m, Mp, Np, Kp, nks, mtiles, ntiles, count;
    int Rp, rtiles;    // residue scheme: B columns padded to 256, and their tiles
    int residues_ok;   // the plane block has room for the residue scheme
    size_t sc_per_leaf, dg_per_leaf, sc_base, dg_base, total;
    size_t off_fa, off_fb, off_ea, off_la, off_eb, off_lb;  // within a scalar block
    size_t off_da, off_db;                                  // digit planes
    size_t off_ra, off_rb;                                  // residue planes of A and B
    size_t z_base;                                          // product-residue scratch
};

__host__ __device__ inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

__host__ __device__ inline Geo make_geo(int m, int count, int scheme) {
    Geo g;
    g.m = m;
    g.count = count;
    g.Mp = (m + TM - 1) / TM * TM;
    g.Np = (m + TN - 1) / TN * TN;
    g.Kp = (m + TK - 1) / TK * TK;
    g.nks = g.Kp / TK;
    g.mtiles = g.Mp / TM;
    g.ntiles = g.Np / TN;
    g.Rp = (m + RTN - 1) / RTN * RTN;
    g.rtiles = g.Rp / RTN;
    g.residues_ok = scheme != SCHEME_DIGITS && g.Kp <= RKMAX;
    size_t o = 0;
    g.off_fa = o; o += align256((size_t)g.Mp * 4);
    g.off_fb = o; o += align256((size_t)g.Np * 4);
    g.off_ea = o; o += align256((size_t)g.Mp * 4);
    g.off_la = o; o += align256((size_t)g.Mp * 4);
    g.off_eb = o; o += align256((size_t)g.Np * 4);
    g.off_lb = o; o += align256((size_t)g.Np * 4);
    g.sc_per_leaf = o;
    o = 0;
    g.off_da = o; o += align256((size_t)g.Mp * g.Kp * 2 * MAXS);
    g.off_db = o; o += align256((size_t)g.Np * g.Kp * 2 * MAXS);
    const size_t digits_bytes = o;
    o = 0;
    g.off_ra = o; o += align256((size_t)LMAX * g.Mp * g.Kp * 2);
    g.off_rb = o; o += align256((size_t)LMAX * g.Rp * g.Kp * 2);
    const size_t residue_bytes = o;
    g.dg_per_leaf = g.residues_ok && residue_bytes > digits_bytes ? residue_bytes : digits_bytes;
    g.sc_base = 256;
    g.dg_base = 256 + (size_t)count * g.sc_per_leaf;
    g.z_base = g.dg_base + (size_t)count * g.dg_per_leaf;
    g.total = g.z_base + (g.residues_ok ? (size_t)ZCTA_MAX * 2 * ZTILE_BYTES : 0);
    return g;
}

__device__ __forceinline__ char *leaf_scalars(char *ws, const Geo &g, int l) {
    return ws + g.sc_base + (size_t)l * g.sc_per_leaf;
}
__device__ __forceinline__ char *leaf_digits(char *ws, const Geo &g, int l) {
    return ws + g.dg_base + (size_t)l * g.dg_per_leaf;
}

__device__ __forceinline__ void resolve_sd(const SplitHdr *h, SplitParams p, int &s, int &nd) {
    int need = h->needed;
    if (need < 1) need = 1;
    if (need > MAXS) need = MAXS;
    s = p.slices > 0 ? p.slices : need;
    if (s > MAXS) s = MAXS;
    nd = p.diagonals > 0 ? p.diagonals : (2 * s - 1 < 8 ? 2 * s - 1 : 8);
    if (nd > 2 * s - 1) nd = 2 * s - 1;  // no digit pair lies beyond diagonal 2s
    if (nd > 8) nd = 8;
    if (nd < 1) nd = 1;
}

// exponent bound E (|x| < 2^E) and lowest set bit of x != 0, from the two
// 32-bit halves of the encoding: on GB300 64-bit integer operations (shifts,
// 64-bit find-first-set) go to the FP64 pipe, which runs at 1/64 rate and
// held the exponent scan to about half the copy rate.
__device__ __forceinline__ void exp_lsb(double x, int &E, int &lsb) {
    const uint32_t hi = (uint32_t)__double2hiint(x), lo = (uint32_t)__double2loint(x);
    const int field = (int)((hi >> 20) & 0x7FFu);
    const uint32_t mh = (hi & 0xFFFFFu) | (field ? 0x100000u : 0u);  // significand bits 32..52
    const int ctz = lo ? __ffs((int)lo) - 1 : 32 + __ffs((int)mh) - 1;
    E = field ? field - 1022 : -1022;
    lsb = (field ? field : 1) - 1075 + ctz;
}

// x != 0 from its encoding with 32-bit operations (an FP64 compare runs at
// 1/64 rate)
__device__ __forceinline__ bool nonzero_bits(double x) {
    return (((uint32_t)__double2hiint(x) << 1) | (uint32_t)__double2loint(x)) != 0u;
}

// round(x 2^f) to nearest, ties to even, for |x 2^f| <= 2^55, by integer
// operations on the IEEE bits (the FP64 pipe runs at 1/64 of FP32 here).
// With x = +-M 2^e (M < 2^53) and f = t - E, t <= 55, E >= e + 52 (E = -1022
// and M < 2^52 for subnormals), the shift e + f is at most 3 and M << 3 stays
// below 2^56, so a left shift never overflows.
__device__ __forceinline__ long long scaled_round(double x, int f) {
    unsigned long long u = (unsigned long long)__double_as_longlong(x);
    int field = (int)((u >> 52) & 0x7ff);
    unsigned long long M = u & 0xFFFFFFFFFFFFFull;
    int e;
    if (field == 0) {
        if (M == 0) return 0;
        e = -1074;
    } else {
        M |= 1ull << 52;
        e = field - 1075;
    }
    int sh = e + f;
    unsigned long long q;
    if (sh >= 0) {
        q = M << sh;
    } else {
        int r = -sh;
        if (r > 63) {
            q = 0;
        } else {
            q = M >> r;
            unsigned long long rem = M & ((1ull << r) - 1), half = 1ull << (r - 1);
            if (rem > half || (rem == half && (q & 1))) q++;
        }
    }
    return (u >> 63) ? -(long long)q : (long long)q;
}

// ---------------------------------------------------------------- sm_100+ wrappers
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait: false (and a status bit) if the phase never completes
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, unsigned *status,
                                          unsigned code, uint32_t limit = WAIT_LIMIT) {
    for (uint32_t it = 0; it < limit; it++) {
        if (mbar_try(bar, parity)) return true;
        if (it > 64) __nanosleep(it > 4096 ? 256 : 32);
    }
    atomicOr(status, code);
    return false;
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes,
                                         uint32_t bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            dst),
        "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}

// UMMA shared-memory descriptor, K-major, no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
    return d;                // base offset 0, swizzle none
}

// instruction descriptor: kind::f16, A=B=bf16, D=f32, K-major, M x N
__device__ __forceinline__ uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc,
                                     uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
        : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
          "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
          "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]),
          "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]),
          "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

}  // namespace split
}  // namespace caps
