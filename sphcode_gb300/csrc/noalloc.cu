// Energy and momentum sums over caller-owned device arrays without any device allocation.
//
// The library's own sums (sphgpu_energy, integrate.cu) reduce through a partial-sum buffer that
// the context allocates.  Some callers cannot allocate device memory at the point where they
// need the sums: host programs that hand out all device memory themselves from a pool fixed at
// start-up (a cudaMalloc behind the pool's back fails or breaks its accounting), and loops that
// must not stall the device (cudaMalloc and cudaFree can synchronise it).  This variant keeps its
// scratch in a file-scope __device__ array instead, so every GPU that loads the library holds
// that array (NOALLOC_MAX_CHUNKS * NOALLOC_SUMS doubles, 229,376 bytes) until the process exits.
#include <cuda.h>

#include <mutex>
#include <string>

#include "context.cuh"

namespace sphgpu {

namespace {

constexpr int NOALLOC_CHUNK = 8192;          // particles per partial sum
constexpr int NOALLOC_MAX_CHUNKS = 4096;     // => at most 33,554,432 particles per call
constexpr int NOALLOC_SUMS = 7;              // kinetic, thermal, potential, unused, p_x, p_y, p_z
constexpr int NOALLOC_THREADS = 256;
constexpr int MAX_DEVICES = 64;

// The scratch: one row of NOALLOC_SUMS partial sums per chunk.  Host code must not pass the
// name of this array to a kernel (on the host it is only a stand-in); the kernels receive its
// device address, looked up once per device with cudaGetSymbolAddress.
static __device__ __align__(256) double noalloc_scratch[NOALLOC_MAX_CHUNKS * NOALLOC_SUMS];

// Looked-up device addresses, keyed by device and by the CUDA context current at the lookup (a
// context created anew, e.g. after cudaDeviceReset, loads the module again at a new address).
std::mutex g_addr_mutex;
struct ScratchAddr {
    CUcontext ctx;
    double* addr;
};
ScratchAddr g_scratch_addr[MAX_DEVICES] = {};
// Pass 1: chunk c of the particles writes its sums to row c (every row read by pass 2 is
// written by pass 1 of the same call, so nothing has to start at zero).
__global__ void noalloc_partial_kernel(int dim, int n, const double* mass, const double* vel,
                                       const double* ene, const double* phi, double* partial)
{
    const int chunk = blockIdx.x;
    const int b = chunk * NOALLOC_CHUNK, e = min(n, b + NOALLOC_CHUNK);
    double s[NOALLOC_SUMS] = {0, 0, 0, 0, 0, 0, 0};
    for (int i = b + threadIdx.x; i < e; i += blockDim.x) {
        const double m = mass[i];
        double v2 = 0.0;
        for (int k = 0; k < dim; ++k) {
            const double v = vel[(size_t)i * dim + k];
            v2 += v * v;
            s[4 + k] += m * v;
        }
        s[0] += 0.5 * m * v2;
        s[1] += m * ene[i];
        if (phi) s[2] += 0.5 * m * phi[i];
    }
    __shared__ double red[NOALLOC_SUMS][NOALLOC_THREADS / 32];
    for (int q = 0; q < NOALLOC_SUMS; ++q) {
        double v = s[q];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
        if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x < NOALLOC_SUMS) {
        double v = 0.0;
        for (int w = 0; w < NOALLOC_THREADS / 32; ++w) v += red[threadIdx.x][w];
        partial[(size_t)chunk * NOALLOC_SUMS + threadIdx.x] = v;
    }
}

// Pass 2: the partials of all chunks in a fixed order (deterministic), written to the caller's
// output {kinetic, thermal, potential, total, p_0 .. p_{dim-1}}.  Thread t sums the chunks
// t, t + 256, ... in turn; the 256 thread sums are then added pairwise in a fixed tree.
__global__ void noalloc_final_kernel(int dim, int nchunks, const double* partial, double* out)
{
    __shared__ double red[NOALLOC_SUMS][NOALLOC_THREADS];
    double s[NOALLOC_SUMS] = {0, 0, 0, 0, 0, 0, 0};
    for (int c = threadIdx.x; c < nchunks; c += NOALLOC_THREADS)
        for (int q = 0; q < NOALLOC_SUMS; ++q) s[q] += partial[(size_t)c * NOALLOC_SUMS + q];
    for (int q = 0; q < NOALLOC_SUMS; ++q) red[q][threadIdx.x] = s[q];
    __syncthreads();
    for (int w = NOALLOC_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int q = 0; q < NOALLOC_SUMS; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = red[0][0];
        out[1] = red[1][0];
        out[2] = red[2][0];
        out[3] = red[0][0] + red[1][0] + red[2][0];
        for (int k = 0; k < dim; ++k) out[4 + k] = red[4 + k][0];
    }
}

using CtxGetCurrentFn = CUresult (*)(CUcontext*);

// The context current on the calling thread (NULL when none is, or the driver entry point is
// unavailable).
CUcontext current_context()
{
    static CtxGetCurrentFn fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            f = nullptr;
        }
        return reinterpret_cast<CtxGetCurrentFn>(f);
    }();
    CUcontext ctx = nullptr;
    if (fn && fn(&ctx) != CUDA_SUCCESS) ctx = nullptr;
    return ctx;
}

// Device address of the scratch on the current device, looked up with cudaGetSymbolAddress on
// the first call per device (and again when the device's context changed since).
int scratch_address(double** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        set_global_error(std::string("sphgpu_energy_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
        return SPHGPU_ERR_NO_DEVICE;
    }
    if (dev < 0 || dev >= MAX_DEVICES) {
        set_global_error("sphgpu_energy_noalloc: device " + std::to_string(dev) + " is beyond the " +
                         std::to_string(MAX_DEVICES) + " devices this entry point keeps addresses for");
        return SPHGPU_ERR_ARG;
    }
    std::lock_guard<std::mutex> lk(g_addr_mutex);
    ScratchAddr& a = g_scratch_addr[dev];
    const CUcontext ctx = current_context();
    if (!a.addr || !ctx || ctx != a.ctx) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, noalloc_scratch);   // also makes the primary context current
        if (e != cudaSuccess) {
            set_global_error(std::string("sphgpu_energy_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            cudaGetLastError();
            return SPHGPU_ERR_CUDA;
        }
        a.addr = static_cast<double*>(p);
        a.ctx = current_context();
    }
    *out = a.addr;
    return SPHGPU_OK;
}

}  // namespace

}  // namespace sphgpu

extern "C" int sphgpu_energy_noalloc(int dim, int n, const double* mass, const double* vel,
                                     const double* ene, const double* phi, double* out,
                                     void* stream)
{
    using namespace sphgpu;
    if (dim < 1 || dim > 3 || n < 1 || !mass || !vel || !ene || !out) {
        set_global_error("sphgpu_energy_noalloc: invalid argument (dim 1..3, n >= 1, non-NULL arrays)");
        return SPHGPU_ERR_ARG;
    }
    if (n > NOALLOC_MAX_CHUNKS * NOALLOC_CHUNK) {
        set_global_error("sphgpu_energy_noalloc: n = " + std::to_string(n) +
                         " exceeds the fixed scratch capacity of " +
                         std::to_string(NOALLOC_MAX_CHUNKS * NOALLOC_CHUNK) + " particles");
        return SPHGPU_ERR_CAPACITY;
    }
    const int nchunks = (n + NOALLOC_CHUNK - 1) / NOALLOC_CHUNK;
    double* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc != SPHGPU_OK) return rc;
    // an error left pending by the caller's earlier work is the caller's: report it, leave it set
    const cudaError_t before = cudaPeekAtLastError();
    if (before != cudaSuccess) {
        set_global_error(std::string("sphgpu_energy_noalloc: a CUDA error from earlier work is pending: ") +
                         cudaGetErrorString(before));
        return SPHGPU_ERR_CUDA;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    noalloc_partial_kernel<<<nchunks, NOALLOC_THREADS, 0, s>>>(dim, n, mass, vel, ene, phi, scratch);
    cudaError_t e = cudaPeekAtLastError();
    if (e == cudaSuccess) {
        noalloc_final_kernel<<<1, NOALLOC_THREADS, 0, s>>>(dim, nchunks, scratch, out);
        e = cudaPeekAtLastError();
    }
    if (e != cudaSuccess) {
        cudaGetLastError();   // raised by this call's launches: clear it
        set_global_error(std::string("sphgpu_energy_noalloc: ") + cudaGetErrorString(e));
        return SPHGPU_ERR_CUDA;
    }
    return SPHGPU_OK;
}
