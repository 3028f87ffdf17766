// nbg_noalloc.cu - all-pairs gravity accelerations on caller-owned device
// buffers with no device allocation at all.
//
// Some callers cannot let a library allocate device memory: a host ODE
// integrator that calls the right-hand side thousands of times per second
// cannot afford cudaMalloc/cudaFree (each can synchronise the device), and a
// process whose device memory belongs to another allocator (for instance the
// pool of a Julia CUDA.jl session that hands out every buffer itself) must not
// have a second allocator take memory behind its back. For them the scratch
// this kernel needs (split positions and per-chunk partial sums) lives in a
// fixed file-scope device array, sized for at most NOALLOC_MAX_BODIES bodies;
// every GPU that loads the library holds that array until the process exits.
#include <mutex>
#include <string>

#include "nbg_internal.cuh"

#define NOALLOC_MAX_BODIES 16384  // multiple of the 512-body i-block
#define NOALLOC_MAX_CHUNKS 8
#define NOALLOC_MAX_DEVICES 64

struct NoallocScratch {
    float4 phi[NOALLOC_MAX_BODIES];
    float4 plo[NOALLOC_MAX_BODIES];
    double part[NOALLOC_MAX_CHUNKS * 3 * NOALLOC_MAX_BODIES];
    unsigned status;
};

// The fixed scratch: sizeof(NoallocScratch) = 3,670,020 bytes per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoallocScratch)];

cudaError_t gravity_raw_launch(const float4* phi, const float4* plo, int64_t n, int64_t npad, int jchunks,
                               double* part, double G, double* a, unsigned* status, cudaStream_t stream);
int gravity_raw_chunks(int device, int64_t npad, int max_chunks);

static std::mutex g_noalloc_mutex;
static NoallocScratch* g_noalloc_addr[NOALLOC_MAX_DEVICES];
static thread_local std::string g_noalloc_err;

const char* noalloc_last_error() { return g_noalloc_err.c_str(); }

// Split positions (hi, lo) with the mass in hi.w; bodies n..npad-1 are the
// far-away massless padding (rewritten on every call: the array keeps the
// previous call's bodies).
__global__ void k_noalloc_pack(const double* __restrict__ x, const double* __restrict__ m, int64_t n, int64_t npad,
                               NoallocScratch* s)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npad; i += (int64_t)gridDim.x * blockDim.x) {
        if (i < n) {
            float h[3], l[3];
            for (int k = 0; k < 3; ++k) {
                double p = x[3 * i + k];
                h[k] = (float)p;
                l[k] = (float)(p - (double)h[k]);
            }
            s->phi[i] = make_float4(h[0], h[1], h[2], (float)m[i]);
            s->plo[i] = make_float4(l[0], l[1], l[2], 0.0f);
        } else {
            s->phi[i] = make_float4(1e18f, 1e18f, 1e18f, 0.0f);
            s->plo[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
}

static int noalloc_fail(int code, const std::string& msg)
{
    g_noalloc_err = msg;
    return code;
}

extern "C" int nbg_gravity_accel_noalloc(const double* x, const double* mass, int64_t n, double G, double* a,
                                         void* stream)
{
    if (!x || !mass || !a || n < 1) return noalloc_fail(NBG_ERR_ARG, "null buffer or n < 1");
    if (n > NOALLOC_MAX_BODIES)
        return noalloc_fail(NBG_ERR_CAPACITY, "nbg_gravity_accel_noalloc: n = " + std::to_string(n) +
                                                  " exceeds the fixed scratch of " +
                                                  std::to_string(NOALLOC_MAX_BODIES) + " bodies");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return noalloc_fail(NBG_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return noalloc_fail(NBG_ERR_UNSUPPORTED, "device index too large");
    NoallocScratch* s = nullptr;
    {
        // once per device, with that device current: the host-side name of a
        // __device__ array is not a device address, so ask the runtime for it
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (!g_noalloc_addr[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess)
                return noalloc_fail(NBG_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_noalloc_addr[dev] = (NoallocScratch*)p;
        }
        s = g_noalloc_addr[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t npad = ((n + 511) / 512) * 512;
    const int jchunks = gravity_raw_chunks(dev, npad, NOALLOC_MAX_CHUNKS);
    e = cudaMemsetAsync(&s->status, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return noalloc_fail(NBG_ERR_CUDA, std::string("status clear: ") + cudaGetErrorString(e));
    k_noalloc_pack<<<grid_for(npad, 256), 256, 0, st>>>(x, mass, n, npad, s);
    e = cudaGetLastError();
    if (e != cudaSuccess) return noalloc_fail(NBG_ERR_CUDA, std::string("k_noalloc_pack: ") + cudaGetErrorString(e));
    e = gravity_raw_launch(s->phi, s->plo, n, npad, jchunks, s->part, G, a, &s->status, st);
    if (e != cudaSuccess) return noalloc_fail(NBG_ERR_CUDA, std::string("k_gravity: ") + cudaGetErrorString(e));
    unsigned w = 0;
    e = cudaMemcpyAsync(&w, &s->status, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return noalloc_fail(NBG_ERR_CUDA, std::string("sync: ") + cudaGetErrorString(e));
    if (w & ST_NONFINITE) return noalloc_fail(NBG_ERR_NONFINITE, "non-finite acceleration");
    return NBG_OK;
}
