// Host engine of the CAPS GB300 multiply: plans the Strassen-Winograd
// recursion for one GPU and launches the kernels; implements the C ABI of
// include/caps_gb300.h.
//
// Reference structure it replaces (one rank): multiply() multiply.cpp:9-25,
// multiplyInternal :28-108, strassenDFS :313-455, strassenBFS :212-310,
// block_multiply :1082-1141, memory budget memory.cpp:4-37, counters
// counters.cpp.
//
// Execution model.  The recursion works on a BATCH of independent
// same-size products.  A 'b' level forms the operand sums of every product of
// the batch in one launch and recurses on a batch seven times larger (the 7
// subproducts run concurrently), then forms C in one launch (calcCij).  A 'd'
// level forms the operand sums once and recurses seven times on a batch of
// the same size, folding each subproduct into C as soon as it is ready, in
// the reference's summation order.  The leaf level runs one batched GEMM
// launch.  Workspace comes from a stack over one device arena; the plan is
// built twice (a dry run sizes the arena, then the real one), and all task
// tables of a call go to the device in one copy.
#include "common.cuh"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <functional>
#include <unordered_map>
#include <mutex>
#include <string>
#include <vector>

#include <sys/stat.h>

namespace caps {

// ------------------------------------------------------------------ state
static thread_local std::string g_last_err;
static std::recursive_mutex g_mu;
std::recursive_mutex &library_mutex() { return g_mu; }
static long long g_launches = 0;
static caps_counters g_counters;
static int g_fail_allocs = 0;
static bool g_phase_timing = false;

void note_cuda_error(cudaError_t e, const char *where) {
    g_last_err = std::string(cudaGetErrorString(e)) + " (" + where + ")";
}
void set_last_error_text(const char *msg) { g_last_err = msg; }
void count_launch(long long n) { g_launches += n; }

static caps_status dev_malloc(void **p, size_t bytes) {
    if (g_fail_allocs > 0) {
        g_fail_allocs--;
        g_last_err = "device allocation failed (injected)";
        return CAPS_ERR_ALLOC;
    }
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        note_cuda_error(e, "cudaMalloc");
        *p = nullptr;
        return CAPS_ERR_ALLOC;
    }
    return CAPS_OK;
}

struct DevBuf {
    char *ptr = nullptr;
    size_t size = 0;
    int device = -1;
};

static caps_status ensure(DevBuf &b, size_t bytes) {
    int dev = 0;
    CAPS_CUDA_TRY(cudaGetDevice(&dev));
    if (b.ptr && b.size >= bytes && b.device == dev) return CAPS_OK;
    if (b.ptr) {
        cudaDeviceSynchronize();
        cudaFree(b.ptr);
        b.ptr = nullptr;
        b.size = 0;
    }
    size_t want = bytes < 256 ? 256 : bytes;
    CAPS_TRY(dev_malloc((void **)&b.ptr, want));
    b.size = want;
    b.device = dev;
    return CAPS_OK;
}

static DevBuf g_arena;   // workspace + task tables
static DevBuf g_io;      // device copies for caps_multiply_host
static DevBuf g_status;  // device status words of split kernels
static DevBuf g_chol;    // -B^T and the product of caps_chol_mult_dev
static DevBuf g_rect;    // task table of caps_rect_mm_dev

struct PinnedBuf {
    void *ptr = nullptr;
    size_t size = 0;
    cudaEvent_t done = nullptr;
    bool pending = false;
};
static PinnedBuf g_pinned;

static caps_status pinned_reserve(size_t bytes) {
    if (g_pinned.pending) {
        CAPS_CUDA_TRY(cudaEventSynchronize(g_pinned.done));
        g_pinned.pending = false;
    }
    if (!g_pinned.done) CAPS_CUDA_TRY(cudaEventCreateWithFlags(&g_pinned.done, cudaEventDisableTiming));
    if (g_pinned.ptr && g_pinned.size >= bytes) return CAPS_OK;
    if (g_pinned.ptr) cudaFreeHost(g_pinned.ptr);
    g_pinned.ptr = nullptr;
    size_t want = std::max<size_t>(bytes, 1 << 16);
    CAPS_CUDA_TRY(cudaMallocHost(&g_pinned.ptr, want));
    g_pinned.size = want;
    return CAPS_OK;
}

// ------------------------------------------------------------------ plan
enum OpKind { K_EW = 0, K_LEAF_DMMA, K_LEAF_SPLIT, K_REORDER, K_WAIT, K_RECORD };

// Events the host entry point uses to overlap its copies with a top-level
// 'd' step: the step waits for A11/B11 (0) before Q1, for A12/B21 (1) before
// Q2 and for the other input quadrants (2) before forming T4/S4; it records
// when C11 (3), C22 (4) and C21 (5) are final, so their copies back run under
// the later subproducts, and C12, the last, in four parts (6..9): its final
// sum runs as four launches, and each part's copy back runs under the next.
constexpr int C12_PARTS = 4;
constexpr int EV_C_FIRST = 3;  // events 3..5: C11, C22, C21 final; 6..9: the parts of C12
// With a level below the top step, its first subproduct Q1 = A11 B11 runs as
// an overlapped lean step too, on the sub-quadrants of A11 and B11: events
// EV_INNER (A11's and B11's first sub-quadrants), +1 (A11's 12 and B11's 21),
// +2 (the rest of A11 and B11).
constexpr int EV_INNER = 6 + C12_PARTS;
// The top step's Q5 = T5 S5 needs A11, A21, B12 and B22 only: it runs once
// A21, B12 and B22 are in (event EV_Q5), before A22, the last copy.
constexpr int EV_Q5 = EV_INNER + 3;
constexpr int HOST_EVENTS = EV_Q5 + 1;

// Part k of C12's q elements: [c12_part_begin(q, k), c12_part_begin(q, k + 1)),
// boundaries on even elements so that the parts keep 16-byte alignment.
static int64_t c12_part_begin(int64_t q, int k) {
    return k >= C12_PARTS ? q : (q * k / C12_PARTS) & ~(int64_t)1;
}
enum Phase { PH_ADD = 0, PH_MUL = 1, PH_REARRANGE = 2 };

struct Op {
    int kind;
    int ew;
    bool vec;
    int64_t q;
    int count;
    size_t toff;   // task table offset in the blob
    size_t toff2;  // second table (reorder dst)
    int m;
    int bs;
    int nrec;
    bool to_caps;
    size_t split_off;  // workspace offset of the split scratch
    SplitParams sp;
    int tile;          // K_LEAF_DMMA: CTA tile shape (DmmaTile)
};

struct Prob {
    const double *A;
    const double *B;
    double *C;
};

struct Builder {
    std::vector<Op> ops;
    std::vector<uint8_t> blob;
    char *ws_base = nullptr;
    size_t top = 0, peak = 0;
    int64_t bs = 1;
    caps_options opt;
    long long adds = 0, muls = 0, add_bytes = 0;
    int split_group = 0;
    bool host_overlap = false;  // emit K_WAIT / K_RECORD at the top-level 'd' step
    int overlap_stage = 0;      // 0: top step not built yet; 1: building its Q1; 2: no more waits
    bool overlap_extras = true; // the overlapped top step's one-pass sums and early Q5 (about
                                // 10 quarter buffers more; dropped when the budget is short)
    int hybrid = 1;             // subproducts an 'h' step runs at once (desc.nproc_summa)

    size_t mark() const { return top; }
    void release(size_t m) { top = m; }
    double *alloc(int64_t elems) {
        size_t off = (top + 255) & ~(size_t)255;
        top = off + (size_t)elems * sizeof(double);
        peak = std::max(peak, top);
        return reinterpret_cast<double *>(ws_base + off);
    }
    size_t alloc_bytes(size_t bytes) {
        size_t off = (top + 255) & ~(size_t)255;
        top = off + bytes;
        peak = std::max(peak, top);
        return off;
    }
    template <typename T>
    size_t table(const std::vector<T> &v) {
        size_t off = (blob.size() + 63) & ~(size_t)63;
        blob.resize(off + v.size() * sizeof(T));
        if (!v.empty()) memcpy(blob.data() + off, v.data(), v.size() * sizeof(T));
        return off;
    }
};

static bool aligned16(const void *p) { return ((uintptr_t)p & 15) == 0; }

static void emit_ew(Builder &b, int op, const std::vector<EwTask> &tasks, int64_t q) {
    bool vec = (q % 2) == 0;
    int ns = ew_sources(op), nd = ew_dests(op);
    for (const EwTask &t : tasks) {
        for (int k = 0; k < ns; k++) vec = vec && aligned16(t.src[k]);
        for (int k = 0; k < nd; k++) vec = vec && aligned16(t.dst[k]);
    }
    {
        // algorithmic bytes: the sources each formula reads plus its outputs
        int reads = ns;
        if (op >= EW_FORM_T4S4 && op <= EW_FORM_T6) reads = (op == EW_FORM_T4S4) ? 6 : 4;
        b.add_bytes += (long long)(reads + nd) * q * 8 * (long long)tasks.size();
    }
    Op o{};
    o.kind = K_EW;
    o.ew = op;
    o.vec = vec;
    o.q = q;
    o.count = (int)tasks.size();
    o.toff = b.table(tasks);
    b.ops.push_back(o);
}

static void emit_event(Builder &b, int kind, int index) {
    Op o{};
    o.kind = kind;
    o.count = index;
    b.ops.push_back(o);
}

// Split-form scratch of one launch group: the slice planes of its leaves
// (285 MB per residue-scheme leaf of 2048) and fixed parts.  Larger groups
// give the persistent GEMMs more work units to balance over the SMs.
static const size_t kSplitGroupBytes = (size_t)16 << 30;

// One batched DMMA launch over m x m leaves, each task with its epilogue fold.
static void emit_dmma(Builder &b, const std::vector<DmmaTask> &t, int64_t m) {
    Op o{};
    o.kind = K_LEAF_DMMA;
    o.count = (int)t.size();
    o.m = (int)m;
    o.tile = b.opt.plain_tile;
    o.toff = b.table(t);
    b.ops.push_back(o);
}

static void emit_leaf_gemm(Builder &b, const std::vector<Prob> &P, int64_t m) {
    if (b.opt.form == CAPS_FORM_SPLIT) {
        // bound split scratch: groups of leaves (the grid's z extent bounds
        // the count too); per leaf = the marginal bytes, over the fixed part
        const int scheme = b.opt.split_scheme;
        const size_t one = split_workspace_bytes((int)m, 1, scheme);
        const size_t per = split_workspace_bytes((int)m, 2, scheme) - one, fixed = one - per;
        const size_t room = kSplitGroupBytes > fixed ? kSplitGroupBytes - fixed : per;
        int g = (int)std::max<size_t>(1, std::min<size_t>(P.size(), room / std::max<size_t>(per, 1)));
        g = std::min(g, 65535);
        if (b.split_group > 0) g = std::min(g, b.split_group);
        // balanced groups: 49 leaves at most 24 to a group run as 17 + 16 + 16,
        // not 24 + 24 + 1 (a short last group leaves most SMs idle)
        const size_t ngroups = (P.size() + g - 1) / g;
        g = (int)((P.size() + ngroups - 1) / ngroups);
        for (size_t s = 0; s < P.size(); s += g) {
            size_t e = std::min(P.size(), s + g);
            std::vector<LeafTask> t;
            for (size_t i = s; i < e; i++) t.push_back({P[i].A, P[i].B, P[i].C});
            Op o{};
            o.kind = K_LEAF_SPLIT;
            o.count = (int)t.size();
            o.m = (int)m;
            o.toff = b.table(t);
            size_t mk = b.mark();
            o.split_off = b.alloc_bytes(split_workspace_bytes((int)m, o.count, scheme));
            b.release(mk);  // scratch is dead once the launch group has run
            // keep the peak: the alloc above already raised it
            o.sp.slices = b.opt.slices;
            o.sp.diagonals = b.opt.diagonals;
            o.sp.scheme = scheme;
            o.sp.bits = b.opt.operand_bits;
            b.ops.push_back(o);
        }
    } else {
        std::vector<DmmaTask> t;
        for (const Prob &p : P) t.push_back(DmmaTask{p.A, p.B, p.C, nullptr, nullptr, nullptr, nullptr, FOLD_STORE, 0});
        emit_dmma(b, t, m);
    }
}

static void emit_reorder(Builder &b, const std::vector<const double *> &src,
                         const std::vector<double *> &dst, int64_t m, int64_t bs, bool to_caps,
                         int nrec = 0) {
    Op o{};
    o.kind = K_REORDER;
    o.count = (int)src.size();
    o.m = (int)m;
    o.bs = (int)bs;
    o.nrec = nrec;
    o.to_caps = to_caps;
    o.toff = b.table(src);
    o.toff2 = b.table(dst);
    b.ops.push_back(o);
}

// block_multiply (multiply.cpp:1082-1141): leaves in bs x bs blocks are
// repacked to column-major when 1 < bs < m, multiplied, and unpacked.
static void build_leaf(Builder &b, const std::vector<Prob> &P, int64_t m) {
    long long m3 = (long long)m * m * m;
    b.adds += m3 * (long long)P.size();
    b.muls += m3 * (long long)P.size();
    if (b.bs == 1 || b.bs == m) {
        emit_leaf_gemm(b, P, m);
        return;
    }
    size_t mk = b.mark();
    std::vector<Prob> Q;
    std::vector<const double *> sa, sb, sc_src;
    std::vector<double *> da, db, sc_dst;
    for (const Prob &p : P) {
        double *w = b.alloc(3 * m * m);
        Q.push_back({w, w + m * m, w + 2 * m * m});
        sa.push_back(p.A);
        da.push_back(w);
        sb.push_back(p.B);
        db.push_back(w + m * m);
        sc_src.push_back(w + 2 * m * m);
        sc_dst.push_back(p.C);
    }
    emit_reorder(b, sa, da, m, b.bs, false);
    emit_reorder(b, sb, db, m, b.bs, false);
    emit_leaf_gemm(b, Q, m);
    emit_reorder(b, sc_src, sc_dst, m, b.bs, true);
    b.release(mk);
}

static void build(Builder &b, const std::vector<Prob> &P, int64_t n, int nrec, const char *pat) {
    if (nrec == 0) {
        build_leaf(b, P, n);
        return;
    }
    const int64_t h = n / 2, q = h * h;
    const char c = pat[0];
    b.adds += 15LL * q * (long long)P.size();
    size_t mk = b.mark();
    std::vector<EwTask> st(P.size());
    const bool hyb = (c == 'h' || c == 'H') && b.hybrid >= 2;
    if (c == 'b' || c == 'B' || hyb) {
        // strassenBFS (multiply.cpp:212-310) on one GPU: 7 subproducts as one
        // batch.  Q1..Q4 are written straight into the C quadrants (calcCij
        // reads all seven products of an element before writing any of its
        // four results), Q5..Q7 into workspace: 11 quarter buffers per node.
        // A hybrid step with factor k (strassenHybrid2..6, multiply.cpp:458-1080,
        // which run k subproducts on k process groups at once) forms the same
        // operands and combines the same products, but runs the subproducts
        // through the levels below k at a time, so only k of them hold
        // workspace at once.
        std::vector<Prob> ch;
        std::vector<EwTask> cij(P.size());
        for (size_t i = 0; i < P.size(); i++) {
            const Prob &p = P[i];
            const double *A11 = p.A, *A21 = p.A + q, *A12 = p.A + 2 * q, *A22 = p.A + 3 * q;
            const double *B11 = p.B, *B21 = p.B + q, *B12 = p.B + 2 * q, *B22 = p.B + 3 * q;
            double *C11 = p.C, *C21 = p.C + q, *C12 = p.C + 2 * q, *C22 = p.C + 3 * q;
            double *W = b.alloc(11 * q);
            double *T3 = W, *T4 = W + q, *T5 = W + 2 * q, *T6 = W + 3 * q;
            double *S3 = W + 4 * q, *S4 = W + 5 * q, *S5 = W + 6 * q, *S7 = W + 7 * q;
            double *Qv[7] = {C11, C12, C21, C22, W + 8 * q, W + 9 * q, W + 10 * q};
            st[i] = EwTask{{A11, A21, A12, A22, B11, B21, B12, B22}, {T3, T4, T5, T6, S3, S4, S5, S7}};
            ch.push_back({A11, B11, Qv[0]});
            ch.push_back({A12, B21, Qv[1]});
            ch.push_back({T3, S3, Qv[2]});
            ch.push_back({T4, S4, Qv[3]});
            ch.push_back({T5, S5, Qv[4]});
            ch.push_back({T6, B22, Qv[5]});
            ch.push_back({A22, S7, Qv[6]});
            EwTask t{};
            for (int k = 0; k < 7; k++) t.src[k] = Qv[k];
            t.dst[0] = C11;
            t.dst[1] = C12;
            t.dst[2] = C21;
            t.dst[3] = C22;
            cij[i] = t;
        }
        emit_ew(b, EW_FORM_ST, st, q);
        if (!hyb) {
            build(b, ch, h, nrec - 1, pat + 1);
        } else {
            // subproducts k at a time; ch holds them node by node, 7 per node
            for (int s0 = 0; s0 < 7; s0 += b.hybrid) {
                std::vector<Prob> part;
                for (size_t i = 0; i < P.size(); i++)
                    for (int k = s0; k < s0 + b.hybrid && k < 7; k++) part.push_back(ch[i * 7 + k]);
                build(b, part, h, nrec - 1, pat + 1);
            }
        }
        emit_ew(b, EW_CALC_CIJ, cij, q);
    } else {
        // strassenDFS (multiply.cpp:409-454), memory-lean: each operand pair
        // is formed just before its subproduct into X, Y, the product goes to
        // Q, and U1 / U2 / U3 live in C quadrants not yet final -- 3 quarter
        // buffers per node.  Per element the sums, products and their order
        // are the reference's:
        //   C11=Q1; C22=C12=U1=C11+Q4; C22=U2=C22+Q5;
        //   C21=U2, C22=U2+Q3, C12=U3=C12+Q3; C21=U2-Q7; C12=U3+Q6; C11+=Q2.
        struct Nd {
            const double *A11, *A21, *A12, *A22, *B11, *B21, *B12, *B22;
            double *C11, *C21, *C12, *C22, *X, *Y, *Q;
        };
        std::vector<Nd> nd(P.size());
        for (size_t i = 0; i < P.size(); i++) {
            const Prob &p = P[i];
            Nd &d = nd[i];
            d.A11 = p.A; d.A21 = p.A + q; d.A12 = p.A + 2 * q; d.A22 = p.A + 3 * q;
            d.B11 = p.B; d.B21 = p.B + q; d.B12 = p.B + 2 * q; d.B22 = p.B + 3 * q;
            d.C11 = p.C; d.C21 = p.C + q; d.C12 = p.C + 2 * q; d.C22 = p.C + 3 * q;
            double *W = b.alloc(3 * q);
            d.X = W; d.Y = W + q; d.Q = W + 2 * q;
        }
        // A step overlapping host copies (below) forms all eight operand sums
        // in one pass once every input is in, into ST = T3 T4 T5 T6 S3 S4 S5
        // S7 (the same formulas as the lean passes: the same bits), and each
        // form() then only points X, Y at its pair.
        double *ST = nullptr;
        auto form = [&](int op) {
            if (ST) {
                Nd &d = nd[0];
                switch (op) {
                    case EW_FORM_T4S4: d.X = ST + q; d.Y = ST + 5 * q; break;
                    case EW_FORM_T5S5: d.X = ST + 2 * q; d.Y = ST + 6 * q; break;
                    case EW_FORM_T3S3: d.X = ST; d.Y = ST + 4 * q; break;
                    case EW_FORM_S7: d.X = ST + 7 * q; break;
                    case EW_FORM_T6: d.X = ST + 3 * q; break;
                }
                return;
            }
            std::vector<EwTask> t(nd.size());
            for (size_t i = 0; i < nd.size(); i++) {
                const Nd &d = nd[i];
                t[i] = EwTask{{d.A11, d.A21, d.A12, d.A22, d.B11, d.B21, d.B12, d.B22}, {d.X, d.Y}};
            }
            emit_ew(b, op, t, q);
        };
        auto sub = [&](int which) {
            std::vector<Prob> ch;
            for (const Nd &d : nd) {
                switch (which) {
                    case 1: ch.push_back({d.A11, d.B11, d.C11}); break;
                    case 2: ch.push_back({d.A12, d.B21, d.Q}); break;
                    case 3: case 4: case 5: ch.push_back({d.X, d.Y, d.Q}); break;
                    case 6: ch.push_back({d.X, d.B22, d.Q}); break;
                    case 7: ch.push_back({d.A22, d.X, d.Q}); break;
                }
            }
            build(b, ch, h, nrec - 1, pat + 1);
        };
        auto comb = [&](int op, auto fill) {
            std::vector<EwTask> t(nd.size());
            for (size_t i = 0; i < nd.size(); i++) {
                t[i] = EwTask{};
                fill(nd[i], t[i]);
            }
            emit_ew(b, op, t, q);
        };
        // At the top of a host call the inputs arrive quadrant by quadrant:
        // Q1 = A11 B11 and Q2 = A12 B21 run first (Q2 into a buffer of its
        // own) while the rest is copied, and C11 = Q1 + Q2 is final as soon as
        // U1 = C11 + Q4 has read Q1 -- the same sums as below, where Q2 comes
        // last to save the buffer.  Stage 0 is that top step: it waits for the
        // input events 0, 1, 2 and records when each C quadrant is final.
        // With a level below, Q1 runs the same way one level down (stage 1,
        // input events EV_INNER..+2 on the sub-quadrants of A11 and B11), so
        // the first products start after a quarter of A11 and B11 is in.
        int stage = -1;
        if (b.host_overlap && P.size() == 1) {
            if (b.overlap_stage == 0 && b.ops.empty()) stage = 0;
            else if (b.overlap_stage == 1) stage = 1;
        }
        const bool top = stage == 0, lead = stage >= 0;
        const int ev = stage == 1 ? EV_INNER : 0;
        double *Q2top = lead ? b.alloc(q) : nullptr;
        if (top && nrec >= 2) {
            // Q1 as a lean step with the sub-quadrant waits (a 'b' and a 'd'
            // step give the same result for the same subproducts)
            char p1[32];
            snprintf(p1, sizeof p1, "%s", pat + 1);
            p1[0] = 'd';
            b.overlap_stage = 1;
            build(b, {{nd[0].A11, nd[0].B11, nd[0].C11}}, h, nrec - 1, p1);
            b.overlap_stage = 2;
        } else {
            if (lead) emit_event(b, K_WAIT, ev);  // A11, B11 on the device
            b.overlap_stage = 2;                  // below this step: no waits
            sub(1);
        }
        double *Q5top = nullptr;
        if (lead) {
            emit_event(b, K_WAIT, ev + 1);  // A12, B21
            build(b, {{nd[0].A12, nd[0].B21, Q2top}}, h, nrec - 1, pat + 1);
        }
        if (lead && b.overlap_extras) {
            ST = b.alloc(8 * q);
            const Nd &d = nd[0];
            if (top) {
                // Q5 = T5 S5 before A22 is in: T5 = A11 - A21, S5 = B22 - B12
                emit_event(b, K_WAIT, EV_Q5);  // A21, B12, B22
                emit_ew(b, EW_FORM_T5S5,
                        {EwTask{{d.A11, d.A21, d.A12, d.A22, d.B11, d.B21, d.B12, d.B22}, {ST + 2 * q, ST + 6 * q}}},
                        q);
                Q5top = b.alloc(q);
                build(b, {{ST + 2 * q, ST + 6 * q, Q5top}}, h, nrec - 1, pat + 1);
            }
            emit_event(b, K_WAIT, ev + 2);  // every input
            emit_ew(b, EW_FORM_ST,
                    {EwTask{{d.A11, d.A21, d.A12, d.A22, d.B11, d.B21, d.B12, d.B22},
                            {ST, ST + q, ST + 2 * q, ST + 3 * q, ST + 4 * q, ST + 5 * q, ST + 6 * q, ST + 7 * q}}},
                    q);
        } else if (lead) {
            emit_event(b, K_WAIT, ev + 2);  // every input; the lean passes form the sums
        }
        // Plain-form leaves right below a step that is not overlapping host
        // copies: each fold that consumes a product (C22 = C12 = C11 + Q4,
        // C22 += Q5, the U2 / Q3 triple, C21 -= Q7, C12 += Q6, C11 += Q2) runs
        // in that product's DMMA epilogue, on the accumulator, instead of as a
        // pass over the stored product: the same FP64 operations in the same
        // order, so the same bits, without the product's round trip to HBM.
        // (Split-form leaves keep the passes: in the residue GEMM's
        // reconstruction warps the folds' FP64 adds slowed the GEMM more than
        // the passes cost.)
        const bool fold = !lead && nrec == 1 && b.opt.form == CAPS_FORM_PLAIN && (b.bs == 1 || b.bs == h);
        auto folded = [&](int which, int mode) {
            std::vector<DmmaTask> t;
            for (const Nd &d : nd) {
                DmmaTask k{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, mode, 0};
                switch (which) {
                    case 2: k.A = d.A12; k.B = d.B21; break;
                    case 3: case 4: case 5: k.A = d.X; k.B = d.Y; break;
                    case 6: k.A = d.X; k.B = d.B22; break;
                    case 7: k.A = d.A22; k.B = d.X; break;
                }
                switch (which) {
                    case 4: k.C = d.C22; k.s0 = d.C11; k.d1 = d.C12; break;                     // ADD_DUP
                    case 5: k.C = d.C22; k.s0 = d.C22; break;                                   // ADD
                    case 3: k.C = d.C21; k.s0 = d.C22; k.s1 = d.C12; k.d1 = d.C22; k.d2 = d.C12; break;  // U2_Q3
                    case 7: k.C = d.C21; k.s0 = d.C21; break;                                   // SUB
                    case 6: k.C = d.C12; k.s0 = d.C12; break;                                   // ADD
                    case 2: k.C = d.C11; k.s0 = d.C11; break;                                   // ADD
                }
                t.push_back(k);
            }
            const long long m3 = (long long)h * h * h * (long long)nd.size();
            b.adds += m3;
            b.muls += m3;
            emit_dmma(b, t, h);
        };
        form(EW_FORM_T4S4);
        if (fold) {
            folded(4, FOLD_ADD_DUP);
        } else {
            sub(4);
            comb(EW_ADD_DUP, [](const Nd &d, EwTask &t) { t.src[0] = d.C11; t.src[1] = d.Q; t.dst[0] = d.C22; t.dst[1] = d.C12; });
        }
        if (lead) {
            comb(EW_ADD, [&](const Nd &d, EwTask &t) { t.src[0] = d.C11; t.src[1] = Q2top; t.dst[0] = d.C11; });
            if (top) emit_event(b, K_RECORD, EV_C_FIRST);  // C11 final
        }
        form(EW_FORM_T5S5);
        if (fold) {
            folded(5, FOLD_ADD);
        } else if (Q5top) {
            comb(EW_ADD, [&](const Nd &d, EwTask &t) { t.src[0] = d.C22; t.src[1] = Q5top; t.dst[0] = d.C22; });
        } else {
            sub(5);
            comb(EW_ADD, [](const Nd &d, EwTask &t) { t.src[0] = d.C22; t.src[1] = d.Q; t.dst[0] = d.C22; });
        }
        form(EW_FORM_T3S3);
        if (fold) {
            folded(3, FOLD_U2_Q3);
        } else {
            sub(3);
            comb(EW_U2_Q3, [](const Nd &d, EwTask &t) { t.src[0] = d.C22; t.src[1] = d.C12; t.src[2] = d.Q; t.dst[0] = d.C21; t.dst[1] = d.C22; t.dst[2] = d.C12; });
        }
        if (top) emit_event(b, K_RECORD, EV_C_FIRST + 1);  // C22 final
        form(EW_FORM_S7);
        if (fold) {
            folded(7, FOLD_SUB);
        } else {
            sub(7);
            comb(EW_SUB, [](const Nd &d, EwTask &t) { t.src[0] = d.C21; t.src[1] = d.Q; t.dst[0] = d.C21; });
        }
        if (top) emit_event(b, K_RECORD, EV_C_FIRST + 2);  // C21 final
        form(EW_FORM_T6);
        if (fold) {
            folded(6, FOLD_ADD);
        } else if (top) {
            sub(6);
            // C12 = U3 + Q6 in parts, each recorded when final
            for (int k = 0; k < C12_PARTS; k++) {
                const int64_t p0 = c12_part_begin(q, k), p1 = c12_part_begin(q, k + 1);
                if (p1 > p0)
                    emit_ew(b, EW_ADD, {EwTask{{nd[0].C12 + p0, nd[0].Q + p0}, {nd[0].C12 + p0}}}, p1 - p0);
                emit_event(b, K_RECORD, EV_C_FIRST + 3 + k);
            }
        } else {
            sub(6);
            comb(EW_ADD, [](const Nd &d, EwTask &t) { t.src[0] = d.C12; t.src[1] = d.Q; t.dst[0] = d.C12; });
        }
        if (fold) {
            folded(2, FOLD_ADD);
        } else if (!lead) {
            sub(2);
            comb(EW_ADD, [](const Nd &d, EwTask &t) { t.src[0] = d.C11; t.src[1] = d.Q; t.dst[0] = d.C11; });
        }
    }
    b.release(mk);
}

// ------------------------------------------------------------------ checks
// nproc_summa is the reference's P factor, the process groups a hybrid step
// spreads its subproducts over; on one GPU it is the number of subproducts an
// 'h' step runs at once (1: the step runs as 'd', as the reference does on one
// rank; 2..6: strassenHybrid2..6's split; other values are rejected, as
// multiply.cpp:92-96 rejects them).
static caps_status check_desc(const caps_desc &d) {
    if (d.nproc != 1 || d.nprocr != 1 || d.nprocc != 1 || d.nproc_summa < 1 || d.nproc_summa > 6)
        return CAPS_ERR_UNSUPPORTED;
    if (d.lda <= 0 || d.nrec < 0 || d.bs <= 0 || d.nrec > 24) return CAPS_ERR_SIZE;
    int64_t unit = ((int64_t)1 << d.nrec) * d.bs;
    if (d.lda % unit != 0) return CAPS_ERR_SIZE;
    return CAPS_OK;
}

static caps_status check_pattern(const caps_desc &d, const char *pat) {
    if (!pat) return CAPS_OK;
    for (int l = 0; l < d.nrec; l++) {
        char c = pat[l];
        if (c == 0) return CAPS_ERR_INVALID_PATTERN;
        if (!(c == 'b' || c == 'B' || c == 'd' || c == 'D' || c == 'h' || c == 'H'))
            return CAPS_ERR_INVALID_PATTERN;
    }
    return CAPS_OK;
}

static caps_options opts_or_default(const caps_options *o) {
    caps_options r;
    caps_options_init(&r);
    if (o) r = *o;
    return r;
}

static caps_status check_opts(const caps_options &o) {
    if (o.form != CAPS_FORM_PLAIN && o.form != CAPS_FORM_SPLIT) return CAPS_ERR_ARG;
    if (o.slices < 0 || o.slices > 8) return CAPS_ERR_ARG;
    if (o.diagonals < 0 || o.diagonals > 8) return CAPS_ERR_ARG;
    if (o.split_scheme < CAPS_SPLIT_AUTO || o.split_scheme > CAPS_SPLIT_RESIDUES) return CAPS_ERR_ARG;
    if (o.plain_tile < CAPS_TILE_64x64 || o.plain_tile > CAPS_TILE_128x64) return CAPS_ERR_ARG;
    if (o.operand_bits < CAPS_OPERAND_BITS_TUNED || o.operand_bits > 55) return CAPS_ERR_ARG;
    return CAPS_OK;
}

// Bytes of workspace one level's pattern char costs for a batch of `count`.
static int64_t level_ws(char c, int64_t n, int64_t count) {
    int64_t q = (n / 2) * (n / 2);
    return (c == 'b' || c == 'B' ? 11 : 3) * q * 8 * count;
}

// Chooses a pattern when the caller gives none: 'b' at the deepest levels
// while the extra workspace fits the budget (batching the subproducts keeps
// the GPU full), 'd' above (memory-lean), as the -m budget drives the BFS
// choice in the reference (multiply.cpp:43-66).
static void auto_pattern(const caps_desc &d, const caps_options &o, char *out) {
    int r = d.nrec;
    for (int l = 0; l < r; l++) out[l] = 'd';
    out[r] = 0;
    int64_t budget = o.workspace_limit > 0 ? o.workspace_limit : ((int64_t)24 << 30);
    for (int l = r - 1; l >= 0; l--) {
        out[l] = 'b';
        // workspace along the recursion: sum over levels of per-level cost
        int64_t total = 0, count = 1, n = d.lda;
        for (int k = 0; k < r; k++) {
            total += level_ws(out[k], n, count);
            if (out[k] == 'b' || out[k] == 'B') count *= 7;
            n /= 2;
        }
        if (o.form == CAPS_FORM_SPLIT)
            total += (int64_t)std::min<size_t>(split_workspace_bytes((int)n, (int)count, o.split_scheme), kSplitGroupBytes);
        if (total > budget) {
            out[l] = 'd';
            break;
        }
    }
}

struct Planned {
    Builder b;
    size_t ws_bytes;
    size_t table_off;
    size_t total;
};

static caps_status plan(const double *A, const double *B, double *C, const caps_desc &d,
                        const char *pat, const caps_options &o, char *ws_base, Planned &pl,
                        bool host_overlap = false, bool overlap_extras = true) {
    pl.b = Builder();
    pl.b.host_overlap = host_overlap;
    pl.b.overlap_extras = overlap_extras;
    pl.b.ws_base = ws_base;
    pl.b.bs = d.bs;
    pl.b.hybrid = d.nproc_summa;
    pl.b.opt = o;
    std::vector<Prob> P{{A, B, C}};
    build(pl.b, P, d.lda, d.nrec, pat);
    pl.ws_bytes = (pl.b.peak + 255) & ~(size_t)255;
    pl.table_off = pl.ws_bytes;
    pl.total = pl.table_off + pl.b.blob.size() + 256;
    return CAPS_OK;
}

// ------------------------------------------------------------------ run
struct KernelTiming {
    double gemm_seconds = 0;   // base-case GEMM kernels only (DMMA or tcgen05)
    long long gemm_launches = 0;
    double gemm_leaf_m3 = 0;   // sum over launches of count * m^3
};

static caps_status upload_tables(const std::vector<uint8_t> &blob, char *dst, cudaStream_t s) {
    if (blob.empty()) return CAPS_OK;
    CAPS_TRY(pinned_reserve(blob.size()));
    memcpy(g_pinned.ptr, blob.data(), blob.size());
    CAPS_CUDA_TRY(cudaMemcpyAsync(dst, g_pinned.ptr, blob.size(), cudaMemcpyHostToDevice, s));
    CAPS_CUDA_TRY(cudaEventRecord(g_pinned.done, s));
    g_pinned.pending = true;
    return CAPS_OK;
}

// Streams and events of the host entry points, one set per device (a call
// made with another device current must not record on the first device's
// stream or events).  Created on first use on a device, destroyed by
// caps_release_cache.
struct HostSide {
    int device = -1;
    cudaStream_t copy = nullptr;             // H2D / D2H copies beside the multiply
    cudaEvent_t start = nullptr;             // earlier work on the caller's stream is done
    cudaEvent_t c_ready = nullptr;           // caps_chol_mult_host: C is on the device
    cudaEvent_t events[HOST_EVENTS] = {};    // caps_multiply_host: quadrant hand-offs
    cudaEvent_t timing[5] = {};              // phase timing: start, first inputs, all inputs,
                                             // compute end, copy-back end
};
static std::deque<HostSide> g_host_sides;  // deque: elements stay put as devices are added

static caps_status host_side(HostSide **out) {
    int dev = 0;
    CAPS_CUDA_TRY(cudaGetDevice(&dev));
    for (HostSide &h : g_host_sides)
        if (h.device == dev) {
            *out = &h;
            return CAPS_OK;
        }
    HostSide h;
    h.device = dev;
    CAPS_CUDA_TRY(cudaStreamCreateWithFlags(&h.copy, cudaStreamNonBlocking));
    CAPS_CUDA_TRY(cudaEventCreateWithFlags(&h.start, cudaEventDisableTiming));
    CAPS_CUDA_TRY(cudaEventCreateWithFlags(&h.c_ready, cudaEventDisableTiming));
    for (int i = 0; i < HOST_EVENTS; i++) CAPS_CUDA_TRY(cudaEventCreateWithFlags(&h.events[i], cudaEventDisableTiming));
    for (int i = 0; i < 5; i++) CAPS_CUDA_TRY(cudaEventCreate(&h.timing[i]));
    g_host_sides.push_back(h);
    *out = &g_host_sides.back();
    return CAPS_OK;
}

// The quadrant events of the host call in progress (K_WAIT / K_RECORD ops).
static cudaEvent_t *g_host_events = nullptr;

// Launches a plan's ops.  `tables`: the plan's task tables on the device;
// `ws_base`: the workspace base its offsets refer to.

static caps_status launch_ops(const std::vector<Op> &ops, char *tables, char *ws_base, cudaStream_t s,
                              double *phase_time, KernelTiming *kt) {
    struct Rec {
        cudaEvent_t e0, e1;
        int phase;
        bool gemm;
        double m3;
    };
    std::vector<Rec> recs;
    auto ev_begin = [&](cudaEvent_t &e) {
        cudaEventCreate(&e);
        cudaEventRecord(e, s);
    };
    for (const Op &o : ops) {
        const bool timed = phase_time || kt;
        Rec r{nullptr, nullptr, PH_ADD, false, 0.0};
        cudaError_t err = cudaSuccess;
        switch (o.kind) {
            case K_EW:
                if (timed) ev_begin(r.e0);
                err = launch_elementwise(o.ew, reinterpret_cast<const EwTask *>(tables + o.toff), o.count, o.q, s, o.vec);
                r.phase = PH_ADD;
                break;
            case K_LEAF_DMMA:
                if (timed) ev_begin(r.e0);
                err = launch_dmma_gemm(reinterpret_cast<const DmmaTask *>(tables + o.toff), o.count, o.m, s, o.tile);
                r.phase = PH_MUL;
                r.gemm = true;
                r.m3 = (double)o.count * o.m * (double)o.m * o.m;
                break;
            case K_LEAF_SPLIT: {
                const LeafTask *t = reinterpret_cast<const LeafTask *>(tables + o.toff);
                void *ws = ws_base + o.split_off;
                // scan + prep are timed with the multiply phase but not as GEMM
                Rec pre{nullptr, nullptr, PH_MUL, false, 0.0};
                if (timed) ev_begin(pre.e0);
                err = launch_split_scan(t, o.count, o.m, o.sp, ws, s);
                if (err == cudaSuccess) err = launch_split_prep(t, o.count, o.m, o.sp, ws, s);
                if (timed) {
                    cudaEventCreate(&pre.e1);
                    cudaEventRecord(pre.e1, s);
                    recs.push_back(pre);
                }
                if (err != cudaSuccess) break;
                if (timed) ev_begin(r.e0);
                err = launch_split_gemm(t, o.count, o.m, o.sp, ws, reinterpret_cast<unsigned *>(g_status.ptr), s);
                r.phase = PH_MUL;
                r.gemm = true;
                r.m3 = (double)o.count * o.m * (double)o.m * o.m;
                break;
            }
            case K_WAIT:
                err = cudaStreamWaitEvent(s, g_host_events[o.count], 0);
                if (err != cudaSuccess) {
                    note_cuda_error(err, "cudaStreamWaitEvent");
                    return CAPS_ERR_CUDA;
                }
                continue;
            case K_RECORD:
                err = cudaEventRecord(g_host_events[o.count], s);
                if (err != cudaSuccess) {
                    note_cuda_error(err, "cudaEventRecord");
                    return CAPS_ERR_CUDA;
                }
                continue;
            case K_REORDER:
                if (timed) ev_begin(r.e0);
                err = launch_reorder(reinterpret_cast<const double *const *>(tables + o.toff),
                                     reinterpret_cast<double *const *>(tables + o.toff2), o.count, o.m, o.nrec,
                                     o.bs, o.to_caps, s);
                r.phase = PH_REARRANGE;
                break;
        }
        if (err != cudaSuccess) {
            note_cuda_error(err, "kernel launch");
            return CAPS_ERR_CUDA;
        }
        if (timed) {
            cudaEventCreate(&r.e1);
            cudaEventRecord(r.e1, s);
            recs.push_back(r);
        }
    }
    if (!recs.empty()) {
        CAPS_CUDA_TRY(cudaStreamSynchronize(s));
        for (Rec &r : recs) {
            float ms = 0;
            cudaEventElapsedTime(&ms, r.e0, r.e1);
            if (phase_time) phase_time[r.phase] += ms * 1e-3;
            if (kt && r.gemm) {
                kt->gemm_seconds += ms * 1e-3;
                kt->gemm_launches += 1;
                kt->gemm_leaf_m3 += r.m3;
            }
            cudaEventDestroy(r.e0);
            cudaEventDestroy(r.e1);
        }
    }
    return CAPS_OK;
}

// Work a caller enqueues once the plan's tables are on their way and before
// its kernels (the host entry point's input copies: queued after the tables,
// they cannot hold the tables' copy up behind gigabytes of inputs).
using AfterUpload = std::function<caps_status()>;

static caps_status run_ops(Planned &pl, cudaStream_t s, double *phase_time, KernelTiming *kt,
                           const AfterUpload &after_upload = nullptr) {
    char *tables = g_arena.ptr + pl.table_off;
    CAPS_TRY(upload_tables(pl.b.blob, tables, s));
    if (after_upload) CAPS_TRY(after_upload());
    return launch_ops(pl.b.ops, tables, g_arena.ptr, s, phase_time, kt);
}

static caps_status status_buffer() {
    if (!g_status.ptr) {
        CAPS_TRY(ensure(g_status, 256));
        CAPS_CUDA_TRY(cudaMemset(g_status.ptr, 0, 256));
    }
    return CAPS_OK;
}

// Reads (and clears) the device status word of the split kernels, and the
// digit / diagonal counts (digit scheme) or the moduli count (residue scheme)
// the last split launch group used.
static caps_status check_device_status(cudaStream_t s, const void *last_split_ws) {
    if (!g_status.ptr) return CAPS_OK;
    unsigned h = 0;
    int sd[4] = {0, 0, 0, 0};  // needed, digits, diagonals, moduli (split header)
    CAPS_CUDA_TRY(cudaMemcpyAsync(&h, g_status.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    if (last_split_ws)
        CAPS_CUDA_TRY(cudaMemcpyAsync(sd, last_split_ws, sizeof sd, cudaMemcpyDeviceToHost, s));
    CAPS_CUDA_TRY(cudaStreamSynchronize(s));
    g_counters.split_moduli = sd[3];
    g_counters.split_slices = sd[3] ? 0 : sd[1];
    g_counters.split_diagonals = sd[3] ? 0 : sd[2];
    if (h != 0) {
        CAPS_CUDA_TRY(cudaMemsetAsync(g_status.ptr, 0, sizeof(unsigned), s));
        char buf[96];
        snprintf(buf, sizeof buf, "device wait gave up (status 0x%x)", h);
        g_last_err = buf;
        return CAPS_ERR_TIMEOUT;
    }
    return CAPS_OK;
}

static caps_status resolve_operand_bits(const caps_desc &d, caps_options &o);

static caps_status multiply_dev_locked(const double *A, const double *B, double *C, caps_desc d,
                                       const char *pattern, const caps_options &o_in, cudaStream_t s,
                                       bool sync_status, bool host_overlap = false,
                                       const AfterUpload &after_upload = nullptr) {
    CAPS_TRY(check_desc(d));
    CAPS_TRY(check_pattern(d, pattern));
    CAPS_TRY(check_opts(o_in));
    caps_options o = o_in;
    CAPS_TRY(resolve_operand_bits(d, o));
    if (!A || !B || !C) return CAPS_ERR_ARG;
    char pat[32];
    if (pattern) {
        for (int l = 0; l < d.nrec; l++) pat[l] = pattern[l];
        pat[d.nrec] = 0;
    } else {
        auto_pattern(d, o, pat);
    }
    Planned pl;
    bool extras = true;
    CAPS_TRY(plan(A, B, C, d, pat, o, nullptr, pl, host_overlap, extras));
    if (host_overlap && o.workspace_limit > 0 && (long long)pl.ws_bytes > o.workspace_limit) {
        extras = false;  // the overlapped top step without its extra buffers
        CAPS_TRY(plan(A, B, C, d, pat, o, nullptr, pl, host_overlap, extras));
    }
    if (o.workspace_limit > 0 && (long long)pl.ws_bytes > o.workspace_limit) {
        g_last_err = "workspace of the pattern exceeds the budget";
        return CAPS_ERR_BUDGET;
    }
    if (o.form == CAPS_FORM_SPLIT) CAPS_TRY(status_buffer());
    CAPS_TRY(ensure(g_arena, pl.total));
    CAPS_TRY(plan(A, B, C, d, pat, o, g_arena.ptr, pl, host_overlap, extras));
    double pt[3] = {0, 0, 0};
    long long l0 = g_launches;
    KernelTiming kt;
    CAPS_TRY(run_ops(pl, s, g_phase_timing ? pt : nullptr, g_phase_timing ? &kt : nullptr, after_upload));
    g_counters.time_leaf_gemm = kt.gemm_seconds;
    g_counters.leaf_gemm_launches = kt.gemm_launches;
    g_counters.leaf_gemm_m3 = kt.gemm_leaf_m3;
    g_counters.additions = pl.b.adds;
    g_counters.multiplications = pl.b.muls;
    g_counters.add_bytes = pl.b.add_bytes;
    g_counters.time_add = pt[PH_ADD];
    g_counters.time_mul = pt[PH_MUL];
    g_counters.time_rearrange = pt[PH_REARRANGE];
    g_counters.workspace_peak_bytes = (long long)pl.ws_bytes;
    g_counters.kernel_launches = g_launches - l0;
    if (o.form == CAPS_FORM_SPLIT && sync_status) {
        const void *last = nullptr;
        for (const Op &op : pl.b.ops)
            if (op.kind == K_LEAF_SPLIT) last = g_arena.ptr + op.split_off;
        CAPS_TRY(check_device_status(s, last));
    }
    return CAPS_OK;
}


// ------------------------------------------------------------------ batched
// Independent multiplies of uneven sizes (column-major in and out).  The
// instances are grouped by size; for each size the autotuner picks the depth,
// b/d pattern, split scheme, DMMA tile and residue operand bits; inputs are
// reordered to CAPS layout on the device, every instance of a size class
// runs in one batched recursion (its base case one persistent GEMM launch per
// launch group), and results are reordered back.
// The whole sequence is captured once as a CUDA graph and replayed while the
// same batch (sizes and pointers) comes back.

struct BatchItem {
    int n;
    const double *A, *B;
    double *C;
};

struct TuneEntry {
    int n, form, slices;
    int nrec;
    char pat[8];
    double seconds;
    int scheme;         // the split scheme asked for (caps_options.split_scheme)
    int chosen_scheme;  // the split scheme that won (the plain form: 0)
    int from_cache;     // 1: read from the on-disk cache, not timed in this process
    int tile;           // plain form: the DMMA tile that won (DmmaTile)
    int bits;           // split form, residues: the operand-bit cap that won (0 = 55)
    int rejected;       // smaller caps that were faster but failed the accuracy gate
};
static std::vector<TuneEntry> g_tune;

struct BatchPlan {
    std::vector<BatchItem> items;
    int form = 0, slices = 0, diagonals = 0, scheme = 0;
    long long limit = 0;
    DevBuf buf;
    std::vector<Op> ops;
    std::vector<uint8_t> blob;
    size_t table_off = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long kernels = 0, adds = 0, muls = 0, add_bytes = 0;
};
static std::vector<BatchPlan *> g_batch_plans;
static cudaStream_t g_cap_stream = nullptr;

static void free_plan(BatchPlan *p) {
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    if (p->buf.ptr) cudaFree(p->buf.ptr);
    delete p;
}

static int max_tune_nrec(int n, int form) {
    int mmin = form == CAPS_FORM_SPLIT ? 192 : 96;
    int r = 0;
    while (r < 3 && (n % (2 << r)) == 0 && (n >> (r + 1)) >= mmin) r++;
    return r;
}

static int64_t batch_ws_per_instance(int n, int nrec, const char *pat, int form, int scheme) {
    int64_t total = nrec > 0 ? (int64_t)3 * n * n * 8 : 0, count = 1, m = n;
    for (int k = 0; k < nrec; k++) {
        total += level_ws(pat[k], m, count);
        if (pat[k] == 'b' || pat[k] == 'B') count *= 7;
        m /= 2;
    }
    // the split scratch's per-leaf bytes (its fixed part is counted once per launch group)
    if (form == CAPS_FORM_SPLIT)
        total += (int64_t)(split_workspace_bytes((int)m, (int)(2 * count), scheme) -
                           split_workspace_bytes((int)m, (int)count, scheme));
    return total;
}

struct ClassCfg {
    int n, nrec;
    char pat[8];
    int scheme;  // split form: the scheme the class runs with (caps_split_scheme)
    int tile;    // plain form: base-case CTA tile (DmmaTile)
    int bits;    // split form, residues: operand-bit cap (0 = 55)
};

// Appends the ops of a batch to the builder.
static void build_batch(Builder &b, const std::vector<BatchItem> &items, const std::vector<ClassCfg> &cfg,
                        long long budget) {
    for (const ClassCfg &c : cfg) {
        std::vector<BatchItem> cls;
        for (const BatchItem &it : items)
            if (it.n == c.n) cls.push_back(it);
        if (cls.empty()) continue;
        int64_t per = std::max<int64_t>(1, batch_ws_per_instance(c.n, c.nrec, c.pat, b.opt.form, b.opt.split_scheme));
        size_t chunk = (size_t)std::max<int64_t>(1, budget / per);
        for (size_t s0 = 0; s0 < cls.size(); s0 += chunk) {
            size_t s1 = std::min(cls.size(), s0 + chunk);
            size_t mk = b.mark();
            std::vector<Prob> P;
            std::vector<const double *> ra, rb, rc_src;
            std::vector<double *> da, db, rc_dst;
            for (size_t i = s0; i < s1; i++) {
                const BatchItem &it = cls[i];
                if (c.nrec == 0) {
                    P.push_back({it.A, it.B, it.C});
                    continue;
                }
                int64_t nn = (int64_t)it.n * it.n;
                double *w = b.alloc(3 * nn);
                P.push_back({w, w + nn, w + 2 * nn});
                ra.push_back(it.A);
                da.push_back(w);
                rb.push_back(it.B);
                db.push_back(w + nn);
                rc_src.push_back(w + 2 * nn);
                rc_dst.push_back(it.C);
            }
            if (c.nrec > 0) {
                emit_reorder(b, ra, da, c.n, 1, true, c.nrec);
                emit_reorder(b, rb, db, c.n, 1, true, c.nrec);
            }
            const int asked = b.opt.split_scheme;
            if (b.opt.form == CAPS_FORM_SPLIT) b.opt.split_scheme = c.scheme;
            const int tile = b.opt.plain_tile, bits = b.opt.operand_bits;
            b.opt.plain_tile = c.tile;
            b.opt.operand_bits = c.bits;
            build(b, P, c.n, c.nrec, c.pat);
            b.opt.split_scheme = asked;
            b.opt.plain_tile = tile;
            b.opt.operand_bits = bits;
            if (c.nrec > 0) emit_reorder(b, rc_src, rc_dst, c.n, 1, false, c.nrec);
            b.release(mk);
        }
    }
}

static caps_status plan_batch(BatchPlan &p, const std::vector<ClassCfg> &cfg, const caps_options &o) {
    long long budget = o.workspace_limit > 0 ? o.workspace_limit : ((long long)48 << 30);
    Builder dry;
    dry.opt = o;
    build_batch(dry, p.items, cfg, budget);
    size_t ws = (dry.peak + 255) & ~(size_t)255;
    size_t total = ws + dry.blob.size() + 256;
    if (!p.buf.ptr || p.buf.size < total) {
        if (p.buf.ptr) cudaFree(p.buf.ptr);
        p.buf = DevBuf();
        CAPS_TRY(ensure(p.buf, total));
    }
    Builder real;
    real.opt = o;
    real.ws_base = p.buf.ptr;
    build_batch(real, p.items, cfg, budget);
    p.ops = real.ops;
    p.blob = real.blob;
    p.table_off = ws;
    p.adds = real.adds;
    p.muls = real.muls;
    p.add_bytes = real.add_bytes;
    return CAPS_OK;
}

// Tuning data: uniform [-1, 1), or with `wide` set the same times 2^k, k
// uniform in [-20, 20] (entries spanning 40 binades, the hard case for a
// truncated operand cut).
__global__ void fill_uniform_kernel(double *p, int64_t n, uint64_t seed, int wide) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t z = (uint64_t)i * 0x9E3779B97F4A7C15ull + seed;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        double v = (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
        if (wide) v = ldexp(v, (int)((z & 0xFFFFu) % 41u) - 20);
        p[i] = v;
    }
}

// Error sums of the tuner's accuracy gate over T instances (C of instance i
// at c + i * cstride, its reference at r + i * nn, (|A||B|) at ab + i *
// cstride): out[0] += sum (c - r)^2, out[1] += sum r^2, out[2] = max over
// entries of |c - r| / (|A||B|) (infinite where c is not a number, or where
// it differs from r on an entry whose |A||B| is 0), out[3] = max |r|.
// out[2], out[3] are non-negative doubles, whose encodings order as the
// values do.
__global__ void tune_error_kernel(const double *__restrict__ c, const double *__restrict__ r,
                                  const double *__restrict__ ab, int64_t nn, int T, int64_t cstride, double *out) {
    double s2 = 0, r2 = 0, md = 0, mr = 0;
    const int64_t total = nn * T;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = k / nn, e = k - i * nn;
        const double y = r[k], d = c[i * cstride + e] - y, ad = fabs(d), w = ab[i * cstride + e];
        s2 += d * d;
        r2 += y * y;
        const double rel = w > 0.0 ? ad / w : (ad > 0.0 ? INFINITY : 0.0);
        md = rel == rel ? fmax(md, rel) : INFINITY;
        mr = fmax(mr, fabs(y));
    }
    for (int o = 16; o; o >>= 1) {
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
        r2 += __shfl_xor_sync(0xffffffffu, r2, o);
        md = fmax(md, __shfl_xor_sync(0xffffffffu, md, o));
        mr = fmax(mr, __shfl_xor_sync(0xffffffffu, mr, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(out, s2);
        atomicAdd(out + 1, r2);
        atomicMax(reinterpret_cast<unsigned long long *>(out + 2), (unsigned long long)__double_as_longlong(md));
        atomicMax(reinterpret_cast<unsigned long long *>(out + 3), (unsigned long long)__double_as_longlong(mr));
    }
}

// |x| of the A and B parts of each instance (3 nn apart, A and B first).
__global__ void tune_abs_kernel(const double *__restrict__ src, double *__restrict__ dst, int64_t nn, int T) {
    const int64_t total = 2 * nn * T;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = k / (2 * nn), e = k - i * 2 * nn, x = i * 3 * nn + e;
        dst[x] = fabs(src[x]);
    }
}

static caps_status run_plan_direct(BatchPlan &p, cudaStream_t s) {
    char *tables = p.buf.ptr + p.table_off;
    CAPS_TRY(upload_tables(p.blob, tables, s));
    return launch_ops(p.ops, tables, p.buf.ptr, s, nullptr, nullptr);
}

// Autotuner: for one size and form, times candidates on a synthetic batch of
// that size and keeps the fastest.  Axes, searched in turn (each at the best
// point of the ones before it):
//   1. recursion depth 0..3 (as the leaves allow) and the b/d pattern of the
//      top step; for the split form with the scheme left to the library, also
//      the operand cut (residues where the leaves fit them, digits);
//   2. plain form: the DMMA CTA tile (64 x 64, 32 x 32, 128 x 64);
//   3. split form, where the residues won: the operand-bit cap, 55 / 52 / 48
//      bits (17 / 16 / 15 moduli at K <= 2048: fewer modular products and
//      residue planes).  A smaller cap is kept only if it is faster and, on
//      the uniform batch and on a wide-range batch (u 2^k, k in [-20, 20]),
//      its error against a split reference (depth 0, 55 bits) is no larger
//      than the plain FP64 form's at the same depth and pattern, both
//      normwise and in the largest entry relative to |A||B| (the measure the
//      accuracy target is stated in).
// The split GEMMs' tiles (residues 128 x 256, digits 128 x 64) are fixed:
// the operand slicers write their planes in those tiles' layout.  The
// choices are kept per process and in an on-disk cache (tune_cache_*).

// On-disk cache of the tuner's choices: one tab-separated line per choice,
// keyed by the tuning version, the device's name and SM count, the size,
// form, slices and asked-for scheme.  The file is CAPS_AUTOTUNE_CACHE if set
// (empty: no disk cache), else $HOME/.cache/caps_gb300/autotune.tsv.  A new
// tuning version (a change of the kernels or axes the choices were made
// with) leaves older lines unused; deleting the file forces new timings.
static const char *kTuneVersion = "caps-tune-4";

static std::string tune_cache_path() {
    const char *e = getenv("CAPS_AUTOTUNE_CACHE");
    if (e) return std::string(e);
    const char *home = getenv("HOME");
    if (!home || !*home) return std::string();
    return std::string(home) + "/.cache/caps_gb300/autotune.tsv";
}

static std::string tune_device_key() {
    int dev = 0;
    cudaDeviceProp prop;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
        cudaGetLastError();
        return std::string();
    }
    std::string name(prop.name);
    for (char &c : name)
        if (c == '\t' || c == ' ') c = '_';
    return name + "/" + std::to_string(prop.multiProcessorCount);
}

// One line of the on-disk cache (tune_cache_store's format): true if it
// holds a usable choice for size n under options o on device `dev`.  Each
// line is parsed on its own, so a short or damaged line costs only itself.
static bool parse_tune_line(const char *line, const std::string &dev, int n, const caps_options &o,
                            TuneEntry &out) {
    char ver[64], dk[256], pat[16];
    int fn, fform, fslices, fscheme, nrec, chosen, tile, bits, rejected;
    double sec;
    if (sscanf(line, "%63s %255s %d %d %d %d %d %15s %d %d %d %d %lf", ver, dk, &fn, &fform, &fslices, &fscheme,
               &nrec, pat, &chosen, &tile, &bits, &rejected, &sec) != 13)
        return false;
    if (strcmp(ver, kTuneVersion) || dev != dk || fn != n || fform != o.form || fslices != o.slices ||
        fscheme != o.split_scheme || nrec < 0 || nrec > 3 || tile < 0 || tile >= DMMA_TILES || bits < 0 ||
        bits > 55 || chosen < CAPS_SPLIT_AUTO || chosen > CAPS_SPLIT_RESIDUES)
        return false;
    // the tuner writes nrec steps of 'b' or 'd' ("-" for none); anything
    // else is a damaged or foreign line
    const size_t plen = strcmp(pat, "-") ? strlen(pat) : 0;
    bool pat_ok = plen == (size_t)nrec;
    for (size_t i = 0; i < plen && pat_ok; i++) pat_ok = pat[i] == 'b' || pat[i] == 'd';
    if (!pat_ok) return false;
    TuneEntry t{n, o.form, o.slices, nrec, {0}, sec, o.split_scheme, chosen, 1, tile, bits, rejected};
    memcpy(t.pat, pat, plen);
    out = t;
    return true;
}

static bool tune_cache_lookup(int n, const caps_options &o, TuneEntry &out) {
    const std::string path = tune_cache_path(), dev = tune_device_key();
    if (path.empty() || dev.empty()) return false;
    FILE *f = fopen(path.c_str(), "r");
    if (!f) return false;
    char line[1024];
    bool found = false;
    TuneEntry t;
    while (fgets(line, sizeof line, f))
        if (parse_tune_line(line, dev, n, o, t)) {
            out = t;
            found = true;  // the last matching line wins
        }
    fclose(f);
    return found;
}

static void tune_cache_store(const TuneEntry &t) {
    const std::string path = tune_cache_path(), dev = tune_device_key();
    if (path.empty() || dev.empty()) return;
    const size_t slash = path.rfind('/');
    if (slash != std::string::npos && slash > 0) {
        // the cache's directory and its parent (e.g. ~/.cache/caps_gb300)
        const std::string dir = path.substr(0, slash);
        struct stat sb;
        if (stat(dir.c_str(), &sb) != 0) {
            const size_t up = dir.rfind('/');
            if (up != std::string::npos && up > 0 && stat(dir.substr(0, up).c_str(), &sb) != 0)
                mkdir(dir.substr(0, up).c_str(), 0755);
            mkdir(dir.c_str(), 0755);
        }
    }
    FILE *f = fopen(path.c_str(), "a");
    if (!f) return;
    fprintf(f, "%s\t%s\t%d\t%d\t%d\t%d\t%d\t%s\t%d\t%d\t%d\t%d\t%.9g\n", kTuneVersion, dev.c_str(), t.n, t.form,
            t.slices, t.scheme, t.nrec, t.pat[0] ? t.pat : "-", t.chosen_scheme, t.tile, t.bits, t.rejected,
            t.seconds);
    fclose(f);
}

static void cfg_from_entry(const TuneEntry &t, ClassCfg &out) {
    out.n = t.n;
    out.nrec = t.nrec;
    memcpy(out.pat, t.pat, sizeof out.pat);
    out.scheme = t.chosen_scheme;
    out.tile = t.tile;
    out.bits = t.bits;
}

// Synthetic batch and timing state of one tune_size call.
struct Tuning {
    int n = 0, T = 0;
    int64_t nn = 0;
    double *data = nullptr;  // instance i: A, B, C at data + 3 nn i (+ nn, + 2 nn)
    double *ref = nullptr;   // the gate's reference products, nn per instance
    double *absd = nullptr;  // |A|, |B| and their product |A||B|, laid out as data
    double *err = nullptr;   // tune_error_kernel's four sums
    std::vector<BatchItem> items, abs_items;
    cudaEvent_t e0 = nullptr, e1 = nullptr;

    ~Tuning() {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        for (double *p : {data, ref, absd, err})
            if (p) cudaFree(p);
    }

    void fill(int wide) {
        fill_uniform_kernel<<<1024, 256>>>(data, 3 * nn * T, 12345 + n, wide);
    }

    // Plans and runs one candidate: with `ms`, three runs and the best of the
    // last two; without, one run (its products are what the gate reads).
    caps_status run(const ClassCfg &c, const caps_options &o, double *ms, const std::vector<BatchItem> *its = nullptr) {
        BatchPlan p;
        p.items = its ? *its : items;
        caps_status st = plan_batch(p, {c}, o);
        double t = 1e30;
        for (int rep = 0; rep < (ms ? 3 : 1) && st == CAPS_OK; rep++) {
            cudaEventRecord(e0, 0);
            st = run_plan_direct(p, 0);
            cudaEventRecord(e1, 0);
            if (cudaEventSynchronize(e1) != cudaSuccess) st = CAPS_ERR_CUDA;
            float x = 0;
            cudaEventElapsedTime(&x, e0, e1);
            if (rep > 0) t = std::min(t, (double)x);
        }
        if (p.buf.ptr) cudaFree(p.buf.ptr);
        if (ms) *ms = t;
        return st;
    }

    // Squared error sum, and the largest entry error relative to |A||B| (the
    // measure the split form's accuracy target is stated in), of the batch's
    // products against `ref`.
    caps_status errors(double &s2, double &maxerr) {
        double h[4] = {0, 0, 0, 0};
        CAPS_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof h, 0));
        tune_error_kernel<<<152 * 4, 256>>>(data + 2 * nn, ref, absd + 2 * nn, nn, T, 3 * nn, err);
        CAPS_CUDA_TRY(cudaGetLastError());
        CAPS_CUDA_TRY(cudaMemcpy(h, err, sizeof h, cudaMemcpyDeviceToHost));
        s2 = h[0];
        maxerr = h[2];
        return CAPS_OK;
    }

    // The accuracy gate of an operand-bit cap (see the tuner's comment).
    caps_status gate(const ClassCfg &base, int bits, const caps_options &o, bool &ok) {
        if (!ref) CAPS_TRY(dev_malloc((void **)&ref, (size_t)nn * T * sizeof(double)));
        if (!err) CAPS_TRY(dev_malloc((void **)&err, 4 * sizeof(double)));
        if (!absd) {
            CAPS_TRY(dev_malloc((void **)&absd, (size_t)3 * nn * T * sizeof(double)));
            for (int i = 0; i < T; i++) {
                double *d = absd + 3 * nn * i;
                abs_items.push_back({n, d, d + nn, d + 2 * nn});
            }
        }
        caps_options oref = o, oplain = o;
        oref.form = CAPS_FORM_SPLIT;
        oref.slices = oref.diagonals = 0;
        oref.split_scheme = CAPS_SPLIT_AUTO;
        oplain.form = CAPS_FORM_PLAIN;
        ClassCfg cref{n, 0, {0}, CAPS_SPLIT_AUTO, DMMA_TILE_64x64, 0};
        ClassCfg cplain = base;
        cplain.scheme = 0;
        cplain.bits = 0;
        cplain.tile = DMMA_TILE_64x64;
        ClassCfg cand = base;
        cand.bits = bits;
        ok = true;
        caps_status st = CAPS_OK;
        ClassCfg cabs{n, 0, {0}, 0, DMMA_TILE_64x64, 0};
        for (int wide = 0; wide < 2 && ok && st == CAPS_OK; wide++) {
            fill(wide);
            // |A||B| of every instance, the scale of each entry's error
            tune_abs_kernel<<<1024, 256>>>(data, absd, nn, T);
            if (cudaGetLastError() != cudaSuccess) st = CAPS_ERR_CUDA;
            if (st == CAPS_OK) st = run(cabs, oplain, nullptr, &abs_items);
            if (st == CAPS_OK) st = run(cref, oref, nullptr);
            for (int i = 0; i < T && st == CAPS_OK; i++)
                if (cudaMemcpyAsync(ref + nn * i, data + 3 * nn * i + 2 * nn, (size_t)nn * sizeof(double),
                                    cudaMemcpyDeviceToDevice, 0) != cudaSuccess)
                    st = CAPS_ERR_CUDA;
            double ps2 = 0, pmax = 0, cs2 = 0, cmax = 0;
            if (st == CAPS_OK) st = run(cplain, oplain, nullptr);
            if (st == CAPS_OK) st = errors(ps2, pmax);
            if (st == CAPS_OK) st = run(cand, o, nullptr);
            if (st == CAPS_OK) st = errors(cs2, cmax);
            ok = cs2 <= ps2 && cmax <= pmax;  // false for a NaN
        }
        fill(0);
        return st;
    }
};

// Choices made for single multiplies' leaves (bits_only) are kept under the
// asked-for scheme plus this offset, apart from the batched classes' ones.
constexpr int kLeafGateKey = 8;

// bits_only: the operand-bit cap alone, for leaves of n run at depth 0 with
// residues (a single multiply's leaves with operand_bits = -1).
static caps_status tune_size(int n, const caps_options &o_in, ClassCfg &out, bool bits_only = false) {
    caps_options o = o_in;
    if (bits_only) o.split_scheme = CAPS_SPLIT_RESIDUES;
    caps_options key = o_in;  // what the choice is kept under
    if (bits_only) key.split_scheme += kLeafGateKey;
    for (const TuneEntry &t : g_tune)
        if (t.n == n && t.form == key.form && t.slices == key.slices && t.scheme == key.split_scheme) {
            cfg_from_entry(t, out);
            return CAPS_OK;
        }
    {
        TuneEntry cached;
        if (tune_cache_lookup(n, key, cached)) {
            g_tune.push_back(cached);
            cfg_from_entry(cached, out);
            return CAPS_OK;
        }
    }
    const int rmax = bits_only ? 0 : max_tune_nrec(n, o.form);
    Tuning tu;
    tu.n = n;
    tu.nn = (int64_t)n * n;
    tu.T = (int)std::max<int64_t>(1, std::min<int64_t>(32, ((int64_t)1 << 27) / tu.nn));
    CAPS_TRY(dev_malloc((void **)&tu.data, (size_t)3 * tu.nn * tu.T * sizeof(double)));
    tu.fill(0);
    for (int i = 0; i < tu.T; i++) {
        double *d = tu.data + 3 * tu.nn * i;
        tu.items.push_back({n, d, d + tu.nn, d + 2 * tu.nn});
    }
    CAPS_CUDA_TRY(cudaEventCreate(&tu.e0));
    CAPS_CUDA_TRY(cudaEventCreate(&tu.e1));
    ClassCfg best{n, 0, {0}, o.split_scheme, DMMA_TILE_64x64, 0};
    double best_t = 1e30;
    caps_status st = CAPS_OK;
    // axis 1: depth, pattern and (split form, scheme left to the library)
    // the operand cut; residues only where the leaves fit them, since they
    // would run as digits otherwise
    const bool both = o.form == CAPS_FORM_SPLIT && o.split_scheme == CAPS_SPLIT_AUTO && o.slices == 0;
    for (int r = 0; r <= rmax && st == CAPS_OK; r++) {
        const int leaf = n >> r;
        for (int sc = 0; sc < (both ? 2 : 1) && st == CAPS_OK; sc++) {
            const int scheme = both ? (sc == 0 ? CAPS_SPLIT_RESIDUES : CAPS_SPLIT_DIGITS) : o.split_scheme;
            if (both && scheme == CAPS_SPLIT_RESIDUES && (leaf + 15) / 16 * 16 > RESIDUE_KMAX) continue;
            for (int variant = 0; variant < (r >= 2 ? 2 : 1) && st == CAPS_OK; variant++) {
                ClassCfg c{n, r, {0}, scheme, DMMA_TILE_64x64, 0};
                for (int k = 0; k < r; k++) c.pat[k] = (variant == 1 && k == 0) ? 'd' : 'b';
                double t = 1e30;
                st = tu.run(c, o, &t);
                if (st == CAPS_OK && t < best_t) {
                    best_t = t;
                    best = c;
                }
            }
        }
    }
    // axis 2: the DMMA tile
    if (o.form == CAPS_FORM_PLAIN)
        for (int tile : {(int)DMMA_TILE_32x32, (int)DMMA_TILE_128x64}) {
            if (st != CAPS_OK) break;
            ClassCfg c = best;
            c.tile = tile;
            double t = 1e30;
            st = tu.run(c, o, &t);
            if (st == CAPS_OK && t < best_t) {
                best_t = t;
                best = c;
            }
        }
    // axis 3: the operand-bit cap of the residues, gated on accuracy
    int rejected = 0;
    const int leaf = n >> best.nrec;
    if (st == CAPS_OK && o.form == CAPS_FORM_SPLIT && best.scheme == CAPS_SPLIT_RESIDUES &&
        (leaf + 15) / 16 * 16 <= RESIDUE_KMAX) {
        std::vector<std::pair<double, int>> faster;
        for (int bits : {52, 48}) {
            ClassCfg c = best;
            c.bits = bits;
            double t = 1e30;
            st = tu.run(c, o, &t);
            if (st != CAPS_OK) break;
            if (t < best_t) faster.push_back({t, bits});
        }
        std::sort(faster.begin(), faster.end());
        for (const auto &fb : faster) {
            if (st != CAPS_OK) break;
            bool ok = false;
            st = tu.gate(best, fb.second, o, ok);
            if (st == CAPS_OK && ok) {
                best.bits = fb.second;
                best_t = fb.first;
                break;
            }
            rejected++;
        }
    }
    if (st != CAPS_OK) return st;
    TuneEntry te{n, o.form, o.slices, best.nrec, {0}, best_t / 1e3 / tu.T, key.split_scheme,
                 o.form == CAPS_FORM_SPLIT ? best.scheme : 0, 0, best.tile, best.bits, rejected};
    memcpy(te.pat, best.pat, sizeof te.pat);
    g_tune.push_back(te);
    tune_cache_store(te);
    out = best;
    return CAPS_OK;
}

// caps_options.operand_bits = -1: the residue scheme's operand-bit cap for
// this multiply's leaves, chosen once per leaf size and kept with the
// autotuner's choices (tune_size, bits_only): 55 bits, or 52 / 48 where they
// are faster and pass the accuracy gate against the FP64 DMMA leaf.  Leaves
// the residues do not run (digits forced, slices given, K above 2048) get 0.
static caps_status resolve_operand_bits(const caps_desc &d, caps_options &o) {
    if (o.operand_bits >= 0) return CAPS_OK;
    o.operand_bits = 0;
    const int m = d.lda >> d.nrec;
    if (o.form != CAPS_FORM_SPLIT || o.slices > 0 || o.split_scheme == CAPS_SPLIT_DIGITS ||
        (m + 15) / 16 * 16 > RESIDUE_KMAX)
        return CAPS_OK;
    CAPS_TRY(status_buffer());
    ClassCfg c{};
    CAPS_TRY(tune_size(m, o, c, true));
    o.operand_bits = c.bits;
    return CAPS_OK;
}

static bool same_batch(const BatchPlan &p, const std::vector<BatchItem> &items, const caps_options &o) {
    if (p.form != o.form || p.slices != o.slices || p.diagonals != o.diagonals || p.scheme != o.split_scheme ||
        p.limit != o.workspace_limit ||
        p.items.size() != items.size())
        return false;
    for (size_t i = 0; i < items.size(); i++)
        if (p.items[i].n != items[i].n || p.items[i].A != items[i].A || p.items[i].B != items[i].B ||
            p.items[i].C != items[i].C)
            return false;
    return true;
}

static caps_status multiply_batched_locked(const std::vector<BatchItem> &items, const caps_options &o,
                                           cudaStream_t stream) {
    BatchPlan *plan = nullptr;
    for (BatchPlan *p : g_batch_plans)
        if (same_batch(*p, items, o)) plan = p;
    if (!plan) {
        std::vector<int> sizes;
        for (const BatchItem &it : items)
            if (std::find(sizes.begin(), sizes.end(), it.n) == sizes.end()) sizes.push_back(it.n);
        std::sort(sizes.begin(), sizes.end());
        std::vector<ClassCfg> cfg;
        if (o.form == CAPS_FORM_SPLIT) CAPS_TRY(status_buffer());
        for (int n : sizes) {
            ClassCfg c;
            CAPS_TRY(tune_size(n, o, c));
            cfg.push_back(c);
        }
        plan = new BatchPlan();
        plan->items = items;
        plan->form = o.form;
        plan->slices = o.slices;
        plan->scheme = o.split_scheme;
        plan->diagonals = o.diagonals;
        plan->limit = o.workspace_limit;
        caps_status st = plan_batch(*plan, cfg, o);
        if (st != CAPS_OK) {
            free_plan(plan);
            return st;
        }
        // tables go up once, outside the graph
        char *tables = plan->buf.ptr + plan->table_off;
        if (!plan->blob.empty())
            CAPS_CUDA_TRY(cudaMemcpy(tables, plan->blob.data(), plan->blob.size(), cudaMemcpyHostToDevice));
        if (!g_cap_stream) CAPS_CUDA_TRY(cudaStreamCreateWithFlags(&g_cap_stream, cudaStreamNonBlocking));
        split_gemm_prepare();
        long long l0 = g_launches;
        CAPS_CUDA_TRY(cudaStreamBeginCapture(g_cap_stream, cudaStreamCaptureModeThreadLocal));
        st = launch_ops(plan->ops, tables, plan->buf.ptr, g_cap_stream, nullptr, nullptr);
        cudaError_t ce = cudaStreamEndCapture(g_cap_stream, &plan->graph);
        if (st != CAPS_OK || ce != cudaSuccess) {
            if (ce != cudaSuccess) note_cuda_error(ce, "cudaStreamEndCapture");
            free_plan(plan);
            return st != CAPS_OK ? st : CAPS_ERR_CUDA;
        }
        plan->kernels = g_launches - l0;
        ce = cudaGraphInstantiate(&plan->exec, plan->graph, 0);
        if (ce != cudaSuccess) {
            note_cuda_error(ce, "cudaGraphInstantiate");
            free_plan(plan);
            return CAPS_ERR_CUDA;
        }
        if (g_batch_plans.size() >= 4) {
            free_plan(g_batch_plans.front());
            g_batch_plans.erase(g_batch_plans.begin());
        }
        g_batch_plans.push_back(plan);
    }
    CAPS_CUDA_TRY(cudaGraphLaunch(plan->exec, stream));
    g_counters.additions = plan->adds;
    g_counters.multiplications = plan->muls;
    g_counters.add_bytes = plan->add_bytes;
    g_counters.kernel_launches = plan->kernels;
    if (o.form == CAPS_FORM_SPLIT) CAPS_TRY(check_device_status(stream, nullptr));
    else CAPS_CUDA_TRY(cudaStreamSynchronize(stream));
    return CAPS_OK;
}

// ------------------------------------------------------------------ rectMM
// The rectangular subproject's rectMM on one rank (rect-class/rectmm.cpp:
// 24-72): a classical recursive blocking, not Strassen.  A (m x k), B (k x n)
// and C (m x n) are in its block layout: at each level a column-major grid of
// blocks (A: divm x divk, B: divk x n_blocks, C: divm x divn), the base blocks
// column-major.  The reference's one-rank DFS walk (rectDFS :53-72) is
// replayed on the host to list its base-case products (localRectMM :47-51,
// beta = 0) in order.  Each overwrites its C block, so a block ends up holding
// the last product written to it: every k block overwrites the one before,
// and as the walk moves C one block (not divm blocks) per column block,
// with divm, divn > 1 neighbouring columns' blocks coincide.  The last product
// of each distinct C block runs, all in one batched DMMA launch; blocks the
// walk never writes keep C's entries.  A BFS step needs more than one rank:
// the reference's process split (rectBFS :75-77) leaves none.
static caps_status rect_check(int m, int n, int k, int r, const char *patt, const int *div, int64_t leaf[3]) {
    if (m <= 0 || n <= 0 || k <= 0 || r < 0 || r > 24) return CAPS_ERR_SIZE;
    if (r > 0 && (!patt || !div)) return CAPS_ERR_ARG;
    int64_t mm = m, nn = n, kk = k;
    for (int l = 0; l < r; l++) {
        const char c = patt[l];
        if (c == 'b' || c == 'B') {
            g_last_err = "rectMM: a BFS step splits the processes, and one rank has none to split";
            return CAPS_ERR_UNSUPPORTED;
        }
        if (c != 'd' && c != 'D') return CAPS_ERR_INVALID_PATTERN;
    }
    for (int l = 0; l < r; l++) {
        const int dm = div[3 * l], dn = div[3 * l + 1], dk = div[3 * l + 2];
        if (dm < 1 || dn < 1 || dk < 1 || mm % dm || nn % dn || kk % dk) return CAPS_ERR_SIZE;
        mm /= dm;
        nn /= dn;
        kk /= dk;
    }
    leaf[0] = mm;
    leaf[1] = nn;
    leaf[2] = kk;
    return CAPS_OK;
}

static void rect_walk(const double *A, const double *B, double *C, int64_t m, int64_t n, int64_t k, int r,
                      const int *div, std::vector<LeafTask> &out) {
    if (r == 0) {
        out.push_back({A, B, C});
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
                rect_walk(Ap, B, Cp, newm, newn, newk, r - 1, div + 3, out);
                Ap += subA;
                Cp += subC;
            }
            B += subB;
        }
        C += subC;
    }
}

static caps_status rect_mm_locked(const double *A, const double *B, double *C, int m, int n, int k, int r,
                                  const char *patt, const int *div, cudaStream_t s) {
    int64_t leaf[3];
    CAPS_TRY(rect_check(m, n, k, r, patt, div, leaf));
    if (!A || !B || !C) return CAPS_ERR_ARG;
    if (leaf[0] > INT32_MAX || leaf[1] > INT32_MAX || leaf[2] > INT32_MAX) return CAPS_ERR_SIZE;
    std::vector<LeafTask> walk;
    rect_walk(A, B, C, m, n, k, r, div, walk);
    std::unordered_map<const double *, size_t> last;  // C block -> its last product
    for (size_t i = 0; i < walk.size(); i++) last[walk[i].C] = i;
    std::vector<uint8_t> blob;
    for (size_t i = 0; i < walk.size(); i++) {
        if (last[walk[i].C] != i) continue;
        const DmmaTask t{walk[i].A, walk[i].B, walk[i].C, nullptr, nullptr, nullptr, nullptr, FOLD_STORE, 0};
        const uint8_t *p = reinterpret_cast<const uint8_t *>(&t);
        blob.insert(blob.end(), p, p + sizeof(DmmaTask));
    }
    const int count = (int)(blob.size() / sizeof(DmmaTask));
    CAPS_TRY(ensure(g_rect, blob.size()));
    CAPS_TRY(upload_tables(blob, g_rect.ptr, s));
    long long l0 = g_launches;
    CAPS_CUDA_TRY(launch_dmma_rect(reinterpret_cast<const DmmaTask *>(g_rect.ptr), count, (int)leaf[0], (int)leaf[1],
                                   (int)leaf[2], s));
    g_counters = caps_counters();
    g_counters.multiplications = (long long)count * leaf[0] * leaf[1] * leaf[2];
    g_counters.additions = g_counters.multiplications;
    g_counters.kernel_launches = g_launches - l0;
    return CAPS_OK;
}

}  // namespace caps

using namespace caps;

// ======================================================================= ABI
extern "C" {

void caps_options_init(caps_options *opt) {
    if (!opt) return;
    memset(opt, 0, sizeof(*opt));
    opt->form = CAPS_FORM_PLAIN;
}

caps_status caps_multiply_dev(const double *A, const double *B, double *C, caps_desc desc,
                              const char *pattern, const caps_options *opt, void *stream) {
    std::lock_guard<std::recursive_mutex> g(g_mu);
    return multiply_dev_locked(A, B, C, desc, pattern, opts_or_default(opt), (cudaStream_t)stream, true);
}

// Host arrays: with a top-level 'd' step (the default when no pattern is
// given) the copies overlap the computation -- A11, B11 first, the other
// input quadrants while Q1 runs, and C22 / C21 / C12 back while the later
// subproducts run (copy stream + events placed in the plan); otherwise all
// inputs go in before and C comes back after.
caps_status caps_multiply_host(const double *A, const double *B, double *C, caps_desc desc,
                               const char *pattern, const caps_options *opt) {
    std::lock_guard<std::recursive_mutex> g(g_mu);
    if (!A || !B || !C) return CAPS_ERR_ARG;
    CAPS_TRY(check_desc(desc));
    CAPS_TRY(check_pattern(desc, pattern));
    caps_options o = opts_or_default(opt);
    CAPS_TRY(check_opts(o));
    char pat[32];
    if (pattern) {
        for (int l = 0; l < desc.nrec; l++) pat[l] = pattern[l];
        pat[desc.nrec] = 0;
    } else {
        auto_pattern(desc, o, pat);
        if (desc.nrec > 0) pat[0] = 'd';  // the lean top step lets the copies overlap
    }
    // the lean 'd' step (and 'h' with factor 1, which runs as 'd') waits on the
    // copies quadrant by quadrant; other top steps take the copies whole
    const bool overlap = desc.nrec > 0 && (pat[0] == 'd' || pat[0] == 'D' ||
                                           ((pat[0] == 'h' || pat[0] == 'H') && desc.nproc_summa == 1));
    size_t nn = (size_t)desc.lda * desc.lda * sizeof(double);
    size_t slot = (nn + 255) & ~(size_t)255;
    CAPS_TRY(ensure(g_io, 3 * slot));
    double *dA = (double *)g_io.ptr, *dB = (double *)(g_io.ptr + slot), *dC = (double *)(g_io.ptr + 2 * slot);
    cudaStream_t s = 0;
    if (!overlap) {
        CAPS_CUDA_TRY(cudaMemcpyAsync(dA, A, nn, cudaMemcpyHostToDevice, s));
        CAPS_CUDA_TRY(cudaMemcpyAsync(dB, B, nn, cudaMemcpyHostToDevice, s));
        CAPS_TRY(multiply_dev_locked(dA, dB, dC, desc, pat, o, s, true));
        CAPS_CUDA_TRY(cudaMemcpyAsync(C, dC, nn, cudaMemcpyDeviceToHost, s));
        CAPS_CUDA_TRY(cudaStreamSynchronize(s));
        return CAPS_OK;
    }
    HostSide *hs = nullptr;
    CAPS_TRY(host_side(&hs));
    cudaStream_t cs = hs->copy;
    cudaEvent_t start = hs->start;
    g_host_events = hs->events;
    const size_t q = nn / 4;  // quadrant bytes: X11, X21, X12, X22 at 0, q, 2q, 3q
    auto h2d = [&](double *dst, const double *src, int quad) {
        return cudaMemcpyAsync((char *)dst + quad * q, (const char *)src + quad * q, q, cudaMemcpyHostToDevice, cs);
    };
    const bool timeline = g_phase_timing;  // where the call's time goes (timing events)
    g_counters.host_first_inputs = g_counters.host_all_inputs = 0;
    g_counters.host_compute_end = g_counters.host_copy_back_end = 0;
    if (timeline) CAPS_CUDA_TRY(cudaEventRecord(hs->timing[0], s));  // the call's start
    // The input copies, enqueued once the plan's tables are queued on s (a
    // copy queued later on s waits behind these in the host-to-device copy
    // engine).  Quadrants X11, X21, X12, X22 at 0, q, 2q, 3q: A11 + B11 (Q1),
    // then A12 + B21 (Q2), then A21, B12, B22 (Q5), then A22.
    // With two or more levels the plan's Q1 waits on the sub-quadrants of A11
    // and B11 (events EV_INNER..+2): 11 and 11, then 12 and 21, then the rest.
    const bool inner = desc.nrec >= 2;
    const size_t q4 = q / 4;
    auto h2d_sub = [&](double *dst, const double *src, int sub) {
        return cudaMemcpyAsync((char *)dst + sub * q4, (const char *)src + sub * q4, q4, cudaMemcpyHostToDevice, cs);
    };
    const AfterUpload inputs = [&]() -> caps_status {
        CAPS_CUDA_TRY(cudaEventRecord(start, s));  // after earlier work on s
        CAPS_CUDA_TRY(cudaStreamWaitEvent(cs, start, 0));
        if (inner) {
            CAPS_CUDA_TRY(h2d_sub(dA, A, 0));
            CAPS_CUDA_TRY(h2d_sub(dB, B, 0));
            CAPS_CUDA_TRY(cudaEventRecord(g_host_events[EV_INNER], cs));
            if (timeline) CAPS_CUDA_TRY(cudaEventRecord(hs->timing[1], cs));
            CAPS_CUDA_TRY(h2d_sub(dA, A, 2));
            CAPS_CUDA_TRY(h2d_sub(dB, B, 1));
            CAPS_CUDA_TRY(cudaEventRecord(g_host_events[EV_INNER + 1], cs));
            CAPS_CUDA_TRY(h2d_sub(dA, A, 1));
            CAPS_CUDA_TRY(h2d_sub(dA, A, 3));
            CAPS_CUDA_TRY(h2d_sub(dB, B, 2));
            CAPS_CUDA_TRY(h2d_sub(dB, B, 3));
            CAPS_CUDA_TRY(cudaEventRecord(g_host_events[EV_INNER + 2], cs));
        } else {
            CAPS_CUDA_TRY(h2d(dA, A, 0));
            CAPS_CUDA_TRY(h2d(dB, B, 0));
            if (timeline) CAPS_CUDA_TRY(cudaEventRecord(hs->timing[1], cs));
        }
        CAPS_CUDA_TRY(cudaEventRecord(g_host_events[0], cs));
        CAPS_CUDA_TRY(h2d(dA, A, 2));
        CAPS_CUDA_TRY(h2d(dB, B, 1));
        CAPS_CUDA_TRY(cudaEventRecord(g_host_events[1], cs));
        CAPS_CUDA_TRY(h2d(dA, A, 1));  // A21, B12, B22: Q5's inputs
        CAPS_CUDA_TRY(h2d(dB, B, 2));
        CAPS_CUDA_TRY(h2d(dB, B, 3));
        CAPS_CUDA_TRY(cudaEventRecord(g_host_events[EV_Q5], cs));
        CAPS_CUDA_TRY(h2d(dA, A, 3));  // A22 last
        CAPS_CUDA_TRY(cudaEventRecord(g_host_events[2], cs));
        if (timeline) CAPS_CUDA_TRY(cudaEventRecord(hs->timing[2], cs));
        return CAPS_OK;
    };
    // the plan's own phase timing would synchronise inside the call and
    // serialise the copies back behind the whole multiply: off here
    g_phase_timing = false;
    caps_status st = multiply_dev_locked(dA, dB, dC, desc, pat, o, s, false, true, inputs);
    g_phase_timing = timeline;
    if (st != CAPS_OK) {
        cudaStreamSynchronize(cs);
        return st;
    }
    if (timeline) CAPS_CUDA_TRY(cudaEventRecord(hs->timing[3], s));
    // C11 (quadrant 0), C22 (3), C21 (1) as they become final, then C12 (2)
    // part by part
    const int quad_of_event[3] = {0, 3, 1};
    for (int e = EV_C_FIRST; e < EV_C_FIRST + 3; e++) {
        CAPS_CUDA_TRY(cudaStreamWaitEvent(cs, g_host_events[e], 0));
        const int quad = quad_of_event[e - EV_C_FIRST];
        CAPS_CUDA_TRY(cudaMemcpyAsync((char *)C + quad * q, (char *)dC + quad * q, q, cudaMemcpyDeviceToHost, cs));
    }
    const int64_t qe = (int64_t)(q / sizeof(double));  // elements per quadrant
    for (int k = 0; k < C12_PARTS; k++) {
        CAPS_CUDA_TRY(cudaStreamWaitEvent(cs, g_host_events[EV_C_FIRST + 3 + k], 0));
        const size_t b0 = (size_t)c12_part_begin(qe, k) * sizeof(double), b1 = (size_t)c12_part_begin(qe, k + 1) * sizeof(double);
        if (b1 > b0)
            CAPS_CUDA_TRY(cudaMemcpyAsync((char *)C + 2 * q + b0, (char *)dC + 2 * q + b0, b1 - b0, cudaMemcpyDeviceToHost, cs));
    }
    if (timeline) CAPS_CUDA_TRY(cudaEventRecord(hs->timing[4], cs));
    if (o.form == CAPS_FORM_SPLIT) CAPS_TRY(check_device_status(s, nullptr));
    CAPS_CUDA_TRY(cudaStreamSynchronize(s));
    CAPS_CUDA_TRY(cudaStreamSynchronize(cs));
    if (timeline) {
        double *out[4] = {&g_counters.host_first_inputs, &g_counters.host_all_inputs, &g_counters.host_compute_end,
                          &g_counters.host_copy_back_end};
        for (int i = 0; i < 4; i++) {
            float ms = 0;
            CAPS_CUDA_TRY(cudaEventElapsedTime(&ms, hs->timing[0], hs->timing[i + 1]));
            *out[i] = ms * 1e-3;
        }
    }
    return CAPS_OK;
}

caps_status caps_to_caps_layout_dev(const double *colmajor, double *caps_out, caps_desc desc, void *stream) {
    CAPS_TRY(check_desc(desc));
    if (!colmajor || !caps_out) return CAPS_ERR_ARG;
    CAPS_CUDA_TRY(launch_reorder_one(colmajor, caps_out, desc.lda, desc.nrec, desc.bs, true, (cudaStream_t)stream));
    return CAPS_OK;
}

caps_status caps_from_caps_layout_dev(const double *caps_in, double *colmajor, caps_desc desc, void *stream) {
    CAPS_TRY(check_desc(desc));
    if (!colmajor || !caps_in) return CAPS_ERR_ARG;
    CAPS_CUDA_TRY(launch_reorder_one(caps_in, colmajor, desc.lda, desc.nrec, desc.bs, false, (cudaStream_t)stream));
    return CAPS_OK;
}

caps_status caps_leaf_gemm_dev(const double *A, const double *B, double *C, int m,
                               const caps_options *opt, void *stream) {
    caps_desc d{m, 0, 1, 1, 1, 1, 1};
    return caps_multiply_dev(A, B, C, d, "", opt, stream);
}

// The Cholesky subproject's update on one rank (cholesky/mult.cpp:11-28 with
// x = 1): C = alpha C - A B^T.  -B^T is formed in the recursive layout (an
// exact negation and transpose), A (-B^T) runs as this library's multiply
// with r levels, and C = alpha C + product is one more pass; with alpha = 0
// the multiply writes C directly and C is never read (dgemm's beta = 0 rule,
// mult.cpp:91-98).
static caps_status chol_mult_locked(double *C, const double *A, const double *B, int n, int x, int r,
                                    double alpha, const char *pattern, const caps_options &o, cudaStream_t s,
                                    cudaEvent_t c_ready = nullptr, const AfterUpload &after_upload = nullptr) {
    if (!A || !B || !C) return CAPS_ERR_ARG;
    if (x != 1) {
        g_last_err = "mult: x > 1 process groups need more than one rank";
        return CAPS_ERR_UNSUPPORTED;
    }
    caps_desc d{n, r, 1, 1, 1, 1, 1};
    CAPS_TRY(check_desc(d));
    CAPS_TRY(check_pattern(d, pattern));
    CAPS_TRY(check_opts(o));
    const size_t nn = (size_t)n * n * sizeof(double), slot = (nn + 255) & ~(size_t)255;
    const bool direct = alpha == 0.0;
    CAPS_TRY(ensure(g_chol, direct ? slot : 2 * slot));
    double *nbt = (double *)g_chol.ptr;
    double *prod = direct ? C : (double *)(g_chol.ptr + slot);
    CAPS_CUDA_TRY(launch_rec_transpose(B, nbt, n, r, true, s));
    CAPS_TRY(multiply_dev_locked(A, nbt, prod, d, pattern, o, s, true, false, after_upload));
    if (!direct) {
        if (c_ready) CAPS_CUDA_TRY(cudaStreamWaitEvent(s, c_ready, 0));  // C's copy, made beside the multiply
        CAPS_CUDA_TRY(launch_scale_add(C, prod, alpha, (int64_t)n * n, s));
    }
    return CAPS_OK;
}

caps_status caps_chol_mult_dev(double *C, const double *A, const double *B, int n, int x, int r, double alpha,
                               const char *pattern, const caps_options *opt, void *stream) {
    std::lock_guard<std::recursive_mutex> g(g_mu);
    return chol_mult_locked(C, A, B, n, x, r, alpha, pattern, opts_or_default(opt), (cudaStream_t)stream);
}

caps_status caps_chol_mult_host(double *C, const double *A, const double *B, int n, int x, int r, double alpha,
                                const char *pattern, const caps_options *opt) {
    std::lock_guard<std::recursive_mutex> g(g_mu);
    if (!A || !B || !C) return CAPS_ERR_ARG;
    if (n <= 0) return CAPS_ERR_SIZE;
    const size_t nn = (size_t)n * n * sizeof(double), slot = (nn + 255) & ~(size_t)255;
    CAPS_TRY(ensure(g_io, 3 * slot));
    double *dA = (double *)g_io.ptr, *dB = (double *)(g_io.ptr + slot), *dC = (double *)(g_io.ptr + 2 * slot);
    cudaStream_t s = 0;
    // C is needed only by the final scale-add: it is copied on a side stream
    // while the product runs
    HostSide *hs = nullptr;
    CAPS_TRY(host_side(&hs));
    cudaStream_t cs = hs->copy;
    cudaEvent_t start = hs->start, c_ready = hs->c_ready;
    const bool copy_c = alpha != 0.0;
    CAPS_CUDA_TRY(cudaMemcpyAsync(dB, B, nn, cudaMemcpyHostToDevice, s));
    CAPS_CUDA_TRY(cudaMemcpyAsync(dA, A, nn, cudaMemcpyHostToDevice, s));
    // C's copy, enqueued once the product's task tables are queued on s: a
    // copy queued on s after it would wait behind its gigabytes in the
    // host-to-device copy engine and hold the product back
    const AfterUpload c_copy = [&]() -> caps_status {
        // after A and B are in (the copies share the host link) and after
        // earlier work on s, so dC is free
        CAPS_CUDA_TRY(cudaEventRecord(start, s));
        CAPS_CUDA_TRY(cudaStreamWaitEvent(cs, start, 0));
        CAPS_CUDA_TRY(cudaMemcpyAsync(dC, C, nn, cudaMemcpyHostToDevice, cs));
        CAPS_CUDA_TRY(cudaEventRecord(c_ready, cs));
        return CAPS_OK;
    };
    caps_status st = chol_mult_locked(dC, dA, dB, n, x, r, alpha, pattern, opts_or_default(opt), s,
                                      copy_c ? c_ready : nullptr, copy_c ? c_copy : AfterUpload());
    if (st != CAPS_OK) {
        cudaStreamSynchronize(cs);
        return st;
    }
    CAPS_CUDA_TRY(cudaMemcpyAsync(C, dC, nn, cudaMemcpyDeviceToHost, s));
    CAPS_CUDA_TRY(cudaStreamSynchronize(s));
    return CAPS_OK;
}

caps_status caps_workspace_size(caps_desc desc, const char *pattern, const caps_options *opt, long long *bytes) {
    std::lock_guard<std::recursive_mutex> g(g_mu);
    CAPS_TRY(check_desc(desc));
    CAPS_TRY(check_pattern(desc, pattern));
    if (!bytes) return CAPS_ERR_ARG;
    caps_options o = opts_or_default(opt);
    CAPS_TRY(check_opts(o));
    char pat[32];
    if (pattern) {
        for (int l = 0; l < desc.nrec; l++) pat[l] = pattern[l];
        pat[desc.nrec] = 0;
    } else {
        auto_pattern(desc, o, pat);
    }
    Planned pl;
    const double *z = reinterpret_cast<const double *>(256);
    CAPS_TRY(plan(z, z, const_cast<double *>(z), desc, pat, o, nullptr, pl));
    *bytes = (long long)pl.ws_bytes;
    return CAPS_OK;
}

caps_status caps_resolve_pattern(caps_desc desc, const char *pattern, const caps_options *opt, char *out, int out_len) {
    CAPS_TRY(check_desc(desc));
    CAPS_TRY(check_pattern(desc, pattern));
    if (!out || out_len < desc.nrec + 1) return CAPS_ERR_ARG;
    caps_options o = opts_or_default(opt);
    if (pattern) {
        for (int l = 0; l < desc.nrec; l++) out[l] = pattern[l];
        out[desc.nrec] = 0;
    } else {
        auto_pattern(desc, o, out);
    }
    return CAPS_OK;
}

void caps_get_counters(caps_counters *out) {
    if (out) *out = g_counters;
}
void caps_reset_counters(void) { memset(&g_counters, 0, sizeof(g_counters)); }
void caps_set_phase_timing(int enable) { g_phase_timing = enable != 0; }

const char *caps_status_string(caps_status s) {
    switch (s) {
        case CAPS_OK: return "ok";
        case CAPS_ERR_INVALID_PATTERN: return "Invalid pattern";
        case CAPS_ERR_SIZE: return "matrix dimension not divisible by 2^nrec*bs";
        case CAPS_ERR_BUDGET: return "workspace exceeds the memory budget";
        case CAPS_ERR_CUDA: return "CUDA error";
        case CAPS_ERR_ALLOC: return "device allocation failed";
        case CAPS_ERR_TIMEOUT: return "device wait timed out";
        case CAPS_ERR_UNSUPPORTED: return "unsupported descriptor (one GPU, one rank)";
        case CAPS_ERR_ARG: return "invalid argument";
    }
    return "unknown status";
}

const char *caps_last_cuda_error(void) { return g_last_err.c_str(); }

caps_status caps_multiply_batched_dev(int count, const double *const *A, const double *const *B,
                                      double *const *C, const int *n, const caps_options *opt,
                                      void *stream) {
    std::lock_guard<std::recursive_mutex> g(g_mu);
    if (count < 0 || (count > 0 && (!A || !B || !C || !n))) return CAPS_ERR_ARG;
    caps_options o = opts_or_default(opt);
    CAPS_TRY(check_opts(o));
    std::vector<BatchItem> items;
    for (int i = 0; i < count; i++) {
        if (n[i] <= 0) return CAPS_ERR_SIZE;
        if (!A[i] || !B[i] || !C[i]) return CAPS_ERR_ARG;
        items.push_back({n[i], A[i], B[i], C[i]});
    }
    if (items.empty()) return CAPS_OK;
    return multiply_batched_locked(items, o, (cudaStream_t)stream);
}

caps_status caps_autotune_entry(int index, int *n, int *form, int *nrec, char *pattern, double *seconds) {
    return caps_autotune_entry_ex(index, n, form, nrec, pattern, nullptr, nullptr, seconds);
}

caps_status caps_autotune_entry_ex(int index, int *n, int *form, int *nrec, char *pattern, int *scheme,
                                   int *from_cache, double *seconds) {
    std::lock_guard<std::recursive_mutex> g(g_mu);
    if (index < 0 || index >= (int)g_tune.size()) return CAPS_ERR_ARG;
    const TuneEntry &t = g_tune[index];
    if (n) *n = t.n;
    if (form) *form = t.form;
    if (nrec) *nrec = t.nrec;
    if (pattern) memcpy(pattern, t.pat, sizeof t.pat);
    if (scheme) *scheme = t.chosen_scheme;
    if (from_cache) *from_cache = t.from_cache;
    if (seconds) *seconds = t.seconds;
    return CAPS_OK;
}

static void tune_info_from_entry(const TuneEntry &t, caps_tune_info *out) {
    memset(out, 0, sizeof *out);
    out->n = t.n;
    out->form = t.form;
    out->nrec = t.nrec;
    memcpy(out->pattern, t.pat, sizeof out->pattern);
    out->pattern[sizeof out->pattern - 1] = 0;
    out->scheme = t.chosen_scheme;
    const int leaf = t.nrec >= 0 && t.nrec < 31 ? t.n >> t.nrec : t.n;
    if (t.form == CAPS_FORM_PLAIN) {
        dmma_tile_shape(t.tile, &out->tile_rows, &out->tile_cols);
    } else if (t.chosen_scheme == CAPS_SPLIT_RESIDUES && (leaf + 15) / 16 * 16 <= RESIDUE_KMAX) {
        out->tile_rows = 128;
        out->tile_cols = 256;
        out->operand_bits = t.bits > 0 ? t.bits : 55;
        out->moduli = crt_moduli_needed(out->operand_bits, leaf);
        out->gate_rejected = t.rejected;
        out->leaf_gate = t.scheme >= kLeafGateKey;
    } else {
        out->tile_rows = 128;
        out->tile_cols = 64;
    }
    out->from_cache = t.from_cache;
    out->seconds = t.seconds;
}

caps_status caps_autotune_info(int index, caps_tune_info *out) {
    std::lock_guard<std::recursive_mutex> g(g_mu);
    if (!out || index < 0 || index >= (int)g_tune.size()) return CAPS_ERR_ARG;
    tune_info_from_entry(g_tune[index], out);
    return CAPS_OK;
}

int caps_debug_tune_cache_line(const char *line, const char *device_key, int n, int form, int slices,
                               int split_scheme, caps_tune_info *out) {
    if (!line || !device_key) return 0;
    caps_options o{};
    o.form = form;
    o.slices = slices;
    o.split_scheme = split_scheme;
    TuneEntry t;
    if (!parse_tune_line(line, device_key, n, o, t)) return 0;
    if (out) tune_info_from_entry(t, out);
    return 1;
}

caps_status caps_rect_mm_dev(const double *A, const double *B, double *C, int m, int n, int k, int r,
                             const char *pattern, const int *div_pattern, void *stream) {
    std::lock_guard<std::recursive_mutex> g(g_mu);
    return rect_mm_locked(A, B, C, m, n, k, r, pattern, div_pattern, (cudaStream_t)stream);
}

caps_status caps_rect_mm_host(const double *A, const double *B, double *C, int m, int n, int k, int r,
                              const char *pattern, const int *div_pattern) {
    std::lock_guard<std::recursive_mutex> g(g_mu);
    int64_t leaf[3];
    CAPS_TRY(rect_check(m, n, k, r, pattern, div_pattern, leaf));
    if (!A || !B || !C) return CAPS_ERR_ARG;
    const size_t ba = (size_t)m * k * sizeof(double), bb = (size_t)k * n * sizeof(double),
                 bc = (size_t)m * n * sizeof(double);
    const size_t oa = 0, ob = (ba + 255) & ~(size_t)255, oc = ob + ((bb + 255) & ~(size_t)255);
    CAPS_TRY(ensure(g_io, oc + bc));
    double *dA = (double *)(g_io.ptr + oa), *dB = (double *)(g_io.ptr + ob), *dC = (double *)(g_io.ptr + oc);
    cudaStream_t s = 0;
    // C too: the blocks the walk never writes keep their entries
    CAPS_CUDA_TRY(cudaMemcpyAsync(dA, A, ba, cudaMemcpyHostToDevice, s));
    CAPS_CUDA_TRY(cudaMemcpyAsync(dB, B, bb, cudaMemcpyHostToDevice, s));
    CAPS_CUDA_TRY(cudaMemcpyAsync(dC, C, bc, cudaMemcpyHostToDevice, s));
    CAPS_TRY(rect_mm_locked(dA, dB, dC, m, n, k, r, pattern, div_pattern, s));
    CAPS_CUDA_TRY(cudaMemcpyAsync(C, dC, bc, cudaMemcpyDeviceToHost, s));
    CAPS_CUDA_TRY(cudaStreamSynchronize(s));
    return CAPS_OK;
}

void caps_debug_fail_allocations(int count) { g_fail_allocs = count > 0 ? count : 0; }

void caps_debug_starve_split_gemm(int count) {
    std::lock_guard<std::recursive_mutex> g(g_mu);
    set_debug_starve(count);
}

void caps_release_cache(void) {
    std::lock_guard<std::recursive_mutex> g(g_mu);
    cudaDeviceSynchronize();
    for (BatchPlan *p : g_batch_plans) free_plan(p);
    g_batch_plans.clear();
    for (DevBuf *b : {&g_arena, &g_io, &g_status, &g_chol, &g_rect}) {
        if (b->ptr) cudaFree(b->ptr);
        *b = DevBuf();
    }
    if (g_pinned.ptr) cudaFreeHost(g_pinned.ptr);
    g_pinned.ptr = nullptr;
    g_pinned.size = 0;
    g_pinned.pending = false;
    int cur = 0;
    cudaGetDevice(&cur);
    for (HostSide &h : g_host_sides) {
        cudaSetDevice(h.device);
        cudaStreamDestroy(h.copy);
        cudaEventDestroy(h.start);
        cudaEventDestroy(h.c_ready);
        for (int i = 0; i < HOST_EVENTS; i++) cudaEventDestroy(h.events[i]);
        for (int i = 0; i < 5; i++) cudaEventDestroy(h.timing[i]);
    }
    g_host_sides.clear();
    g_host_events = nullptr;
    cudaSetDevice(cur);
}

}  // extern "C"
