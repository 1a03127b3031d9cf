// Split-form base case that allocates nothing (caps_leaf_gemm_split_noalloc_dev).
//
// Some callers cannot let a library call cudaMalloc: an application that has
// handed all device memory to its own pool allocator (a cudaMalloc would fail
// or break its accounting), or a code path where the device-wide
// synchronisation of cudaMalloc / cudaFree is not acceptable.  For them this
// entry point runs the same kernels as the split form of caps_leaf_gemm_dev
// (scan, finalize, slice, tcgen05 digit-pair GEMM) with all of its scratch --
// the scale arrays, the digit planes, the one-entry task table and the status
// word -- in the file-scope device array below.  Nothing is allocated: no
// cudaMalloc, no cudaFree, no pinned host staging.
//
// Limits and sharing:
//   - leaves up to NOALLOC_MAX_M x NOALLOC_MAX_M (512); larger m is rejected
//     with CAPS_ERR_SIZE before anything is launched;
//   - every GPU that loads the library holds the array (8.5 MiB) until exit;
//   - all calls share the array and it keeps the last call's contents; each
//     call clears the parts that must start at zero.  Calls that overlap on
//     the GPU (work still queued on two streams) race on it: serialise them;
//   - a call holds the library's lock from its set-up to its status read, so
//     calls from several host threads, and calls beside the library's other
//     entry points, take turns on the host;
//   - the first call on a device resolves the array's device address
//     (cudaGetSymbolAddress) with that device current, and keeps it;
//   - every call reads the kernels' status word back, so it synchronises the
//     stream it is given before returning.
#include "common.cuh"

#include <mutex>

namespace caps {

void set_last_error_text(const char *msg);

}  // namespace caps

namespace {

constexpr int NOALLOC_MAX_M = 512;
// split workspace for one 512 x 512 leaf (8,401,152 B) + task table + status
constexpr size_t NOALLOC_BYTES = (size_t)8704 * 1024;
constexpr size_t TASK_OFF = (size_t)8448 * 1024;    // after the split workspace
constexpr size_t STATUS_OFF = TASK_OFF + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

constexpr int MAX_DEVICES = 64;
static void *g_scratch_addr[MAX_DEVICES];  // guarded by the library lock

__global__ void noalloc_set_task(caps::LeafTask *dst, const double *A, const double *B, double *C) {
    dst->A = A;
    dst->B = B;
    dst->C = C;
}

// Device address of the scratch array on the current device (set up once per
// device, with that device current).  Called with the library lock held.
caps_status scratch_address(void **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        caps::note_cuda_error(e, "cudaGetDevice");
        return CAPS_ERR_CUDA;
    }
    if (dev < 0 || dev >= MAX_DEVICES) return CAPS_ERR_UNSUPPORTED;
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            caps::note_cuda_error(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
            return CAPS_ERR_CUDA;
        }
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return CAPS_OK;
}

}  // namespace

extern "C" caps_status caps_leaf_gemm_split_noalloc_dev(const double *A, const double *B, double *C, int m,
                                                        int slices, int diagonals, void *stream) {
    if (!A || !B || !C) return CAPS_ERR_ARG;
    if (slices < 0 || slices > 8 || diagonals < 0 || diagonals > 8) return CAPS_ERR_ARG;
    if (m <= 0 || m > NOALLOC_MAX_M) {
        caps::set_last_error_text("m exceeds the no-allocation scratch limit of 512");
        return CAPS_ERR_SIZE;
    }
    size_t need = caps::split_workspace_bytes(m, 1, CAPS_SPLIT_DIGITS);
    if (need > TASK_OFF) {
        caps::set_last_error_text("split workspace exceeds the no-allocation scratch array");
        return CAPS_ERR_SIZE;
    }
    // the kernels' per-device set-up (constant tables, attributes) and the
    // status word are shared with the other entry points
    std::lock_guard<std::recursive_mutex> lock(caps::library_mutex());
    void *base = nullptr;
    caps_status st = scratch_address(&base);
    if (st != CAPS_OK) return st;
    char *ws = static_cast<char *>(base);
    caps::LeafTask *task = reinterpret_cast<caps::LeafTask *>(ws + TASK_OFF);
    unsigned *status = reinterpret_cast<unsigned *>(ws + STATUS_OFF);
    cudaStream_t s = (cudaStream_t)stream;
    caps::SplitParams p{};
    p.slices = slices;
    p.diagonals = diagonals;
    p.scheme = CAPS_SPLIT_DIGITS;  // the scratch array is sized for digit planes

    noalloc_set_task<<<1, 1, 0, s>>>(task, A, B, C);
    caps::count_launch();
    CAPS_CUDA_TRY(cudaGetLastError());
    CAPS_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(unsigned), s));
    CAPS_CUDA_TRY(caps::launch_split_scan(task, 1, m, p, ws, s));   // clears header and scales
    CAPS_CUDA_TRY(caps::launch_split_prep(task, 1, m, p, ws, s));
    CAPS_CUDA_TRY(caps::launch_split_gemm(task, 1, m, p, ws, status, s));
    unsigned h = 0;
    CAPS_CUDA_TRY(cudaMemcpyAsync(&h, status, sizeof h, cudaMemcpyDeviceToHost, s));
    CAPS_CUDA_TRY(cudaStreamSynchronize(s));
    if (h != 0) {
        caps::set_last_error_text("device wait gave up in the split GEMM");
        return CAPS_ERR_TIMEOUT;
    }
    return CAPS_OK;
}
