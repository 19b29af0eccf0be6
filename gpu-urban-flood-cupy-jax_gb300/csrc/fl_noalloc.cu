// Allocation-free CFL timestep: fl_stable_timestep_noalloc.
//
// Some callers cannot allocate device memory when they need a timestep: a
// plugin that must draw every byte from its host application's memory pool,
// code that runs while another library is capturing the stream into a CUDA
// graph (where a cudaMalloc would break or fail the capture), or a real-time
// service that allows no allocation after start-up.  This entry point gives
// them the global CFL reduction of stable_timestep_s over caller-owned device
// arrays; its only scratch (one float per block for the block minima and the
// grid's done counter) is the file-scope array below, which every GPU that
// loads the library holds until the process exits.
//
// Host code must not pass `g_cfl_scratch` itself to a kernel: on the host that
// name is only a stand-in, not a device address.  The device address is looked
// up once per device with cudaGetSymbolAddress (on the first call made on that
// device, with it current) and passed to the kernel.
#include <mutex>

#include "fl_device.cuh"

namespace fl {

int set_error(int code, const char *fmt, ...);

constexpr int NOALLOC_MAX_BLOCKS = 4096;
constexpr int NOALLOC_THREADS = 256;
constexpr int NOALLOC_CELLS_PER_BLOCK = 2048;  // each thread reduces up to 8 cells
constexpr int64_t NOALLOC_MAX_CELLS = (int64_t)NOALLOC_MAX_BLOCKS * NOALLOC_CELLS_PER_BLOCK;

// [0]: number of blocks done; [1 + b]: bit pattern of block b's minimum.  16 KB.
static __device__ __align__(256) unsigned int g_cfl_scratch[1 + NOALLOC_MAX_BLOCKS];

// The CFL expression of the solver's own reduction (cfl_local, the
// reference's stable_timestep_s of equations.py:155-178 in float32, correctly
// rounded and uncontracted); cells whose local dt is not finite are skipped.
__global__ void __launch_bounds__(NOALLOC_THREADS) k_dt_noalloc(const float *cl, const float *h, const float *hu,
                                                                const float *hv, int32_t n, float cfl, float g,
                                                                float md, unsigned int *scratch, double *dt_out) {
    float best = CUDART_INF_F;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float local = cfl_local(h[i], hu[i], hv[i], cl[i], cfl, g, md);
        if (isfinite(local) && local < best) best = local;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) best = fminf(best, __shfl_xor_sync(0xffffffffu, best, o));
    __shared__ float wmin[NOALLOC_THREADS / 32];
    __shared__ bool last;
    if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
        float b = wmin[0];
        for (int k = 1; k < NOALLOC_THREADS / 32; ++k) b = fminf(b, wmin[k]);
        scratch[1 + blockIdx.x] = __float_as_uint(b);
        __threadfence();
        last = atomicAdd(&scratch[0], 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    float b = CUDART_INF_F;
    for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x)
        b = fminf(b, __uint_as_float(((volatile unsigned int *)scratch)[1 + k]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) b = fminf(b, __shfl_xor_sync(0xffffffffu, b, o));
    if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = b;
    __syncthreads();
    if (threadIdx.x == 0) {
        float m = wmin[0];
        for (int k = 1; k < NOALLOC_THREADS / 32; ++k) m = fminf(m, wmin[k]);
        *dt_out = (m < CUDART_INF_F) ? (double)m : -1.0;
        scratch[0] = 0u;
    }
}

// Device address of g_cfl_scratch, looked up once per device.
static int scratch_address(unsigned int **out) {
    constexpr int MAX_DEVICES = 64;
    static std::mutex mu;
    static unsigned int *addr[MAX_DEVICES] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(FL_E_NO_DEVICE, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= MAX_DEVICES) return set_error(FL_E_INVALID, "device %d is beyond the supported %d", dev, MAX_DEVICES);
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_cfl_scratch);
        if (e != cudaSuccess) return set_error(FL_E_CUDA, "cudaGetSymbolAddress(g_cfl_scratch): %s", cudaGetErrorString(e));
        addr[dev] = (unsigned int *)p;
    }
    *out = addr[dev];
    return FL_OK;
}

}  // namespace fl

extern "C" FL_API int fl_stable_timestep_noalloc(const float *char_len, const float *h, const float *hu,
                                                 const float *hv, int32_t n, double cfl, double gravity_mps2,
                                                 double min_depth_m, double *dt_out, void *stream) {
    using namespace fl;
    if (!char_len || !h || !hu || !hv || !dt_out) return set_error(FL_E_INVALID, "fl_stable_timestep_noalloc: NULL array");
    if (n < 1) return set_error(FL_E_INVALID, "fl_stable_timestep_noalloc: n must be >= 1");
    if ((int64_t)n > NOALLOC_MAX_CELLS)
        return set_error(FL_E_INVALID, "fl_stable_timestep_noalloc: n = %d exceeds the allocation-free limit of %lld cells",
                         n, (long long)NOALLOC_MAX_CELLS);
    unsigned int *scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(unsigned int), st);  // the done counter starts at zero
    if (e != cudaSuccess) return set_error(FL_E_CUDA, "cudaMemsetAsync: %s", cudaGetErrorString(e));
    const int blocks = (int)((n + NOALLOC_CELLS_PER_BLOCK - 1) / NOALLOC_CELLS_PER_BLOCK);
    k_dt_noalloc<<<blocks, NOALLOC_THREADS, 0, st>>>(char_len, h, hu, hv, n, (float)cfl, (float)gravity_mps2,
                                                     (float)min_depth_m, scratch, dt_out);
    e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(FL_E_CUDA, "k_dt_noalloc launch: %s", cudaGetErrorString(e));
    return FL_OK;
}

// ------------------------------------------------------------------ wait self-test
namespace fl {

// One warp waits on an mbarrier that nothing arrives on, with the same bounded
// wait the surface, batch and GEMM kernels use; it must give up after
// limit_ns and report FL_E_TIMEOUT (the context stays usable).
__global__ void k_wait_selftest(uint64_t limit_ns, int32_t *status, uint64_t *elapsed_ns) {
    __shared__ __align__(8) uint64_t bar;
    const uint32_t b = smem_addr(&bar);
    if (threadIdx.x == 0) {
        mbar_init(b, 1);
        mbar_fence_init();
    }
    __syncwarp();
    const uint64_t t0 = global_ns();
    const bool ok = mbar_wait_bounded(b, 0, limit_ns);
    const uint64_t t1 = global_ns();
    if (threadIdx.x == 0) {
        *status = ok ? FL_OK : FL_E_TIMEOUT;
        *elapsed_ns = t1 - t0;
    }
}

}  // namespace fl

extern "C" FL_API int fl_wait_selftest(double limit_s, int32_t *status, double *elapsed_s) {
    using namespace fl;
    if (!status || !elapsed_s || !(limit_s > 0.0) || limit_s > 5.0)
        return set_error(FL_E_INVALID, "fl_wait_selftest: limit must be in (0, 5] s");
    int32_t *d_status = nullptr;
    uint64_t *d_el = nullptr;
    cudaError_t e = cudaMalloc(&d_status, sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&d_el, sizeof(uint64_t));
    if (e != cudaSuccess) {
        cudaFree(d_status);
        return set_error(FL_E_NOMEM, "fl_wait_selftest: %s", cudaGetErrorString(e));
    }
    k_wait_selftest<<<1, 32>>>((uint64_t)(limit_s * 1e9), d_status, d_el);
    uint64_t el = 0;
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(status, d_status, sizeof(int32_t), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&el, d_el, sizeof(uint64_t), cudaMemcpyDeviceToHost);
    cudaFree(d_status);
    cudaFree(d_el);
    if (e != cudaSuccess) return set_error(FL_E_CUDA, "fl_wait_selftest: %s", cudaGetErrorString(e));
    *elapsed_s = (double)el * 1e-9;
    return FL_OK;
}
