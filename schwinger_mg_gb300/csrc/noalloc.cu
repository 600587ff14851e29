// Dot products for callers that must not allocate device memory.
//
// Some callers cannot call cudaMalloc at the moment they need a reduction:
// a host framework that owns every device byte through its own pool and
// forbids outside allocations, a latency-critical loop where an allocation
// (and the implicit synchronisation it may bring) is not acceptable, or a
// process running under a fixed device-memory budget.  smg_blas_dot_noalloc
// serves them: the caller passes its input vectors and an output buffer, and
// the only scratch the kernel needs (per-block partial sums and one
// completion counter per vector) lives in the file-scope array below, which
// every GPU that loads this library holds until the process exits.
#include "smg_internal.h"
#include "reduce.cuh"

#include <mutex>

namespace {

constexpr int kNoAllocMaxRhs = 16;          // vectors per call
constexpr int kNoAllocBlocksPerRhs = 304;   // 2 blocks per SM of a GB300
constexpr int kNoAllocTicketSlots = 32;     // first 256 bytes hold the counters
constexpr int kNoAllocScratchDoubles = kNoAllocTicketSlots + 2 * kNoAllocBlocksPerRhs * kNoAllocMaxRhs;

// 78,080 bytes per device: counters, then partials[rhs][2][block]
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

// per-device address of g_noalloc_scratch, looked up once per device
std::mutex g_scratch_mutex;
void* g_scratch_addr[64] = {};

// sum_i conj(a_i) b_i for vector blockIdx.y; a and b hold nrhs vectors of n
// complex values one after another
__global__ void __launch_bounds__(256) k_dot_noalloc(const cx<double>* __restrict__ a, const cx<double>* __restrict__ b,
                                                     int64_t n, int nrhs, double* scratch, double* out) {
    const int rhs = blockIdx.y;
    unsigned int* tickets = reinterpret_cast<unsigned int*>(scratch);
    double* partials = scratch + kNoAllocTicketSlots;
    double v[2] = {0.0, 0.0};
    const cx<double>* av = a + (int64_t)rhs * n;
    const cx<double>* bv = b + (int64_t)rhs * n;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.y + threadIdx.y; i < n; i += (int64_t)gridDim.x * blockDim.y) {
        const cx<double> c = cmulc(av[i], bv[i]);
        v[0] += c.re;
        v[1] += c.im;
    }
    // blockDim = (1, 256): one rhs lane per block row, blockIdx.y selects the vector
    block_reduce_finalise<2>(v, partials, tickets, nrhs, FinStore{out, 2});
}

smg_status scratch_address(int device, double** out) {
    if (device < 0 || device >= 64) return SMG_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_addr[device]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return SMG_DEVICE_ERROR;
        g_scratch_addr[device] = p;
    }
    *out = static_cast<double*>(g_scratch_addr[device]);
    return SMG_OK;
}

}  // namespace

extern "C" {

SMG_API smg_status smg_blas_dot_noalloc(const double* a, const double* b, int64_t n, int nrhs, double* out,
                                        void* stream) {
    if (!a || !b || !out || n < 0) return SMG_BAD_ARG;
    if (nrhs < 1 || nrhs > kNoAllocMaxRhs) return SMG_BAD_ARG;  // beyond the scratch: 16 vectors per call
    // an error left by earlier work stays with its owner: report it without launching or clearing it
    if (cudaPeekAtLastError() != cudaSuccess) return SMG_DEVICE_ERROR;
    int device = -1;
    if (cudaGetDevice(&device) != cudaSuccess) return SMG_DEVICE_ERROR;
    double* scratch = nullptr;
    smg_status st = scratch_address(device, &scratch);
    if (st != SMG_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the completion counters must start at zero
    if (cudaMemsetAsync(scratch, 0, kNoAllocTicketSlots * sizeof(double), s) != cudaSuccess) return SMG_DEVICE_ERROR;
    int64_t want = (n + 255) / 256;
    int blocks = (int)(want < 1 ? 1 : (want > kNoAllocBlocksPerRhs ? kNoAllocBlocksPerRhs : want));
    k_dot_noalloc<<<dim3(blocks, nrhs), dim3(1, 256), 0, s>>>(reinterpret_cast<const cx<double>*>(a),
                                                               reinterpret_cast<const cx<double>*>(b), n, nrhs,
                                                               scratch, out);
    if (cudaGetLastError() != cudaSuccess) return SMG_DEVICE_ERROR;
    return SMG_OK;
}

}  // extern "C"
