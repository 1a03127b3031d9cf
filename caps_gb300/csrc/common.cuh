// Shared definitions for the CAPS GB300 kernels and host engine.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "../../include/caps_gb300.h"

namespace caps {

// The lock every entry point holds while it plans, launches and reads back:
// the engine's caches, the kernels' per-device set-up and the status word
// are shared by all calls in the process.
std::recursive_mutex &library_mutex();

// Records the CUDA error text for caps_last_cuda_error().
void note_cuda_error(cudaError_t e, const char *where);

#define CAPS_CUDA_TRY(expr)                                  \
    do {                                                     \
        cudaError_t _e = (expr);                             \
        if (_e != cudaSuccess) {                             \
            ::caps::note_cuda_error(_e, #expr);              \
            return CAPS_ERR_CUDA;                            \
        }                                                    \
    } while (0)

#define CAPS_TRY(expr)                                       \
    do {                                                     \
        caps_status _s = (expr);                             \
        if (_s != CAPS_OK) return _s;                        \
    } while (0)

// Count of kernels this library launched (for the bench's launch count).
void count_launch(long long n = 1);

// ---------------------------------------------------------------------------
// Batched elementwise programs over quarter arrays.
//
// One Strassen-Winograd node reads the quadrants X11, X21, X12, X22 of its A
// and B (offsets 0,1,2,3 times q) and forms the operand sums; after the
// subproducts it forms the C quadrants.  The per-element arithmetic and its
// order are the reference's (multiply.cpp:409-454 and calcCij :195-210).
// ---------------------------------------------------------------------------
enum EwOp : int {
    // forms T3,T4,T5,T6 from A and S3,S4,S5,S7 from B (8 outputs)
    EW_FORM_ST = 0,
    // dst0 = src0 (copy)
    EW_COPY = 1,
    // dst0 = src0 + src1 ; dst1 = dst0  (U1 = Q1+Q4 stored in two buffers)
    EW_ADD_DUP = 2,
    // dst0 = src0 + src1
    EW_ADD = 3,
    // dst0 = src0 - src1
    EW_SUB = 4,
    // dst0 = src0 + src2 ; dst1 = src1 + src2   (C22 = U2+Q3 ; U3 = U3+Q3)
    EW_ADD2 = 5,
    // calcCij: C11..C22 from Q1..Q7 (7 inputs, 4 outputs)
    EW_CALC_CIJ = 6,
    // operand pairs of the memory-lean 'd' step, formed just before their
    // subproduct; src = A11 A21 A12 A22 B11 B21 B12 B22
    EW_FORM_T4S4 = 7,  // dst0 = (A21+A22)-A11, dst1 = B22-(B12-B11)
    EW_FORM_T5S5 = 8,  // dst0 = A11-A21,       dst1 = B22-B12
    EW_FORM_T3S3 = 9,  // dst0 = A21+A22,       dst1 = B12-B11
    EW_FORM_S7 = 10,   // dst0 = (B22-(B12-B11))-B21
    EW_FORM_T6 = 11,   // dst0 = A12-((A21+A22)-A11)
    // dst0 = src0 ; dst1 = src0 + src2 ; dst2 = src1 + src2
    // (C21 = U2 ; C22 = U2 + Q3 ; U3 = U1 + Q3)
    EW_U2_Q3 = 12,
};

struct EwTask {
    const double *src[8];
    double *dst[8];
};

// Launches `op` over `count` tasks of q elements each.  `tasks` is a device
// array.  `vec`: every pointer 16-byte aligned and q even (double2 path).
cudaError_t launch_elementwise(int op, const EwTask *tasks, int count, int64_t q,
                               cudaStream_t stream, bool vec);
cudaError_t launch_elementwise(int op, const EwTask *tasks, int count, int64_t q,
                               cudaStream_t stream);
int ew_sources(int op);
int ew_dests(int op);

// Layout reorder (column-major <-> CAPS layout) for `count` matrices.
cudaError_t launch_reorder(const double *const *src_dev, double *const *dst_dev, int count,
                           int64_t n, int nrec, int64_t bs, bool to_caps, cudaStream_t stream);
cudaError_t launch_reorder_one(const double *src, double *dst, int64_t n, int nrec, int64_t bs,
                               bool to_caps, cudaStream_t stream);
// Transpose (times -1 when `negate`) of an n x n matrix in the recursive
// layout with bs = 1; dst must not overlap src.
cudaError_t launch_rec_transpose(const double *src, double *dst, int64_t n, int nrec, bool negate,
                                 cudaStream_t stream);
// c = alpha * c + p over `count` elements.
cudaError_t launch_scale_add(double *c, const double *p, double alpha, int64_t count, cudaStream_t stream);

// ---------------------------------------------------------------------------
// Base-case GEMMs over a batch of leaves (column-major m x m each).
// ---------------------------------------------------------------------------
struct LeafTask {
    const double *A;
    const double *B;
    double *C;
};

// A DMMA base-case product with the fold of a lean 'd' step that consumes
// it, done in the GEMM's epilogue on the FP64 accumulator (the same FP64
// operation the separate combination pass would do on the stored product,
// so the same bits), per element e with p = (A B)_e:
//   FOLD_STORE    C = p
//   FOLD_ADD      C = s0 + p             (EW_ADD with the product second)
//   FOLD_SUB      C = s0 - p             (EW_SUB)
//   FOLD_ADD_DUP  C = d1 = s0 + p        (EW_ADD_DUP: U1 into C22 and C12)
//   FOLD_U2_Q3    C = s0, d1 = s0 + p, d2 = s1 + p  (EW_U2_Q3; s0 = d1, s1 = d2 may alias)
enum DmmaFold { FOLD_STORE = 0, FOLD_ADD, FOLD_SUB, FOLD_ADD_DUP, FOLD_U2_Q3 };
struct DmmaTask {
    const double *A;
    const double *B;
    double *C;
    const double *s0, *s1;
    double *d1, *d2;
    int fold;
    int pad;
};

// FP64 DMMA GEMM (mma.sync f64): C = A * B for every task, in CTA tiles of
// one of three shapes (an autotuner axis).
enum DmmaTile { DMMA_TILE_64x64 = 0, DMMA_TILE_32x32 = 1, DMMA_TILE_128x64 = 2, DMMA_TILES = 3 };
void dmma_tile_shape(int tile, int *rows, int *cols);
cudaError_t launch_dmma_gemm(const DmmaTask *tasks_dev, int count, int m, cudaStream_t stream,
                             int tile = DMMA_TILE_64x64);
// The same for rectangular leaves: A m x k, B k x n, C m x n (column-major,
// leading dimensions m, k, m).
cudaError_t launch_dmma_rect(const DmmaTask *tasks_dev, int count, int m, int n, int k, cudaStream_t stream,
                             int tile = DMMA_TILE_64x64);

// Split form.  Two schemes share one launch sequence; the kernels agree on
// the scheme through the launch group's header, written on the device after
// the exponent scan (no host round trip):
//   digits   -- balanced base-128 digit slices, digit-pair products
//               (kernels_split.cu);
//   residues -- residues modulo up to 17 small coprime moduli, one product per
//               modulus, exact CRT reconstruction (kernels_crt.cu).
// Workspace per leaf: see split_workspace_bytes().
struct SplitParams {
    int slices;     // digit scheme: digits per operand, 1..8 (0 = from the data)
    int diagonals;  // digit scheme: digit-pair diagonals kept, <= 8, >= slices
    int scheme;     // caps_options.split_scheme: 0 automatic, 1 digits, 2 residues
    int bits;       // residue scheme: cap on the operand bits t_a, t_b (0 = 55); fewer
                    // bits need fewer moduli (an autotuner axis, gated on accuracy)
};
size_t split_workspace_bytes(int m, int count, int scheme);
constexpr int RESIDUE_KMAX = 2048;  // residue scheme: largest leaf K (K 90^2 < 2^24, exact fp32 sums)
// Moduli the residue scheme takes for operands of `bits` bits at inner
// dimension K (0 if more than it has).
int crt_moduli_needed(int bits, int K);
// Computes per-row / per-column scale exponents and the needed digit count.
cudaError_t launch_split_scan(const LeafTask *tasks_dev, int count, int m, SplitParams p, void *workspace,
                             cudaStream_t stream);
// Exponents, the scheme choice, and the operand slices (digit or residue planes).
cudaError_t launch_split_prep(const LeafTask *tasks_dev, int count, int m, SplitParams p,
                              void *workspace, cudaStream_t stream);
// Sets the GEMM kernels' attributes and constant tables (once per device);
// call before a stream capture.
void split_gemm_prepare();
// The tensor-core slice products: the digit-pair GEMM with its exact
// recombination epilogue, or the per-modulus residue GEMM with its CRT
// reconstruction warps.
cudaError_t launch_split_gemm(const LeafTask *tasks_dev, int count, int m, SplitParams p,
                              void *workspace, unsigned int *status_dev, cudaStream_t stream);

// Test hook behind caps_debug_starve_split_gemm: the next `count` split GEMM
// launches issue no copies, so their first bounded waits give up (with a
// short limit: nothing is in flight) and the call returns CAPS_ERR_TIMEOUT.
void set_debug_starve(int count);

// kernels_crt.cu, called by the launchers above
cudaError_t crt_prepare();
cudaError_t launch_crt_resolve(int count, int m, SplitParams p, void *workspace, cudaStream_t stream);
cudaError_t launch_crt_slice(const LeafTask *tasks_dev, int count, int m, SplitParams p, void *workspace,
                             cudaStream_t stream);
cudaError_t launch_crt_gemm(const LeafTask *tasks_dev, int count, int m, SplitParams p, void *workspace,
                            unsigned int *status_dev, int num_sms, cudaStream_t stream, int starve = 0);

}  // namespace caps
