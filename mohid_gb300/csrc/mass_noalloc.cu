// mass_noalloc.cu -- compensated mass budget that allocates no memory.
//
// Some callers cannot allocate device memory at the point where they need a
// mass budget: a model whose device memory is owned by another allocator (a
// caching allocator that has already reserved the GPU, or a fixed budget
// reserved when the model starts), or code that runs in the middle of a time
// step where an allocation would synchronise the device or fail under memory
// pressure.  For them this file provides the budget with its scratch in a
// file-scope device array: the CUDA module holding it is loaded (lazily, by
// the first call on a device), and from then on that GPU holds these 128 KiB
// (2 x 8192 doubles) until the process exits.  That first call may therefore
// synchronise or fail under memory pressure like any module load; make it at
// start-up (a warm-up call), outside any time step or stream capture.  Later
// calls call no allocator.
//
// The sum is the Neumaier-compensated FP64 sum of VolumeZ * PROP over water
// cells of the work box (WaterPoints3D == 1), as the batched form's budget:
// one block per j-row writes a compensated partial (sum, correction) into the
// scratch array, and one thread adds the partials in row order, so the result
// does not depend on scheduling.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/mohid_ad.h"
#include "instance.hpp"

namespace {

constexpr int kMaxRows = 8192;                 // largest JUB - 1 (work-box rows) accepted
constexpr int kMaxDevices = 64;
constexpr int kThreads = 256;                  // threads of k_row_mass (its shared arrays)

// scratch of every call on a device: (sum, correction) per j-row
static __device__ __align__(256) double g_row_partials[2 * kMaxRows];

__device__ __forceinline__ void neu_add(double& s, double& c, double x)
{
    const double t = s + x;
    if (fabs(s) >= fabs(x)) c += (s - t) + x; else c += (x - t) + s;
    s = t;
}

// one block per row j = 1..nj: cells (i = 1..ni, k = 1..nk) of the Size-box arrays
__global__ void k_row_mass(const double* __restrict__ P, const double* __restrict__ V,
                           const int* __restrict__ WP, int ni, int nj, int nk, double* partials)
{
    __shared__ double ss[kThreads], sc[kThreads];
    const int j = 1 + blockIdx.x;
    const long long NI = ni + 2, sk = NI * (nj + 2);
    double s = 0.0, c = 0.0;
    const int n = ni * nk;
    for (int e = threadIdx.x; e < n; e += kThreads) {
        const int i = 1 + e % ni, k = 1 + e / ni;
        const long long a = i + NI * j + sk * k;
        if (WP[a] == 1) neu_add(s, c, V[a] * P[a]);
    }
    ss[threadIdx.x] = s;
    sc[threadIdx.x] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        double S = 0.0, C = 0.0;
        for (int q = 0; q < kThreads; ++q) { neu_add(S, C, ss[q]); C += sc[q]; }
        partials[2 * blockIdx.x] = S;
        partials[2 * blockIdx.x + 1] = C;
    }
}

__global__ void k_rows_finish(const double* partials, int nrows, double* out)
{
    double S = 0.0, C = 0.0;
    for (int q = 0; q < nrows; ++q) { neu_add(S, C, partials[2 * q]); C += partials[2 * q + 1]; }
    *out = S + C;
}

// Device address of g_row_partials, looked up once per CUDA context (the
// context's unique id, cuCtxGetId, never reused): after a primary-context reset
// (cudaDeviceReset) or under another context on the same device the module is
// loaded again, at another address, and the lookup is made again.
std::mutex g_mu;
struct ScratchSlot {
    unsigned long long ctx = 0;                // 0: not looked up
    double* p = nullptr;
};
ScratchSlot g_scratch[kMaxDevices];

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// unique id of the calling thread's current context; a thread with no current
// context gets the runtime's primary context of `dev` made current first (the
// runtime would do the same at its first launch)
int current_context_id(int dev, unsigned long long* id, std::string& why)
{
    static CtxGetCurrentFn getCur = nullptr;
    static CtxGetIdFn getId = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            getCur = reinterpret_cast<CtxGetCurrentFn>(p);
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            getId = reinterpret_cast<CtxGetIdFn>(p);
    });
    if (!getCur || !getId) { why = "cuCtxGetCurrent / cuCtxGetId not available"; return MOHID_AD_ERR_CUDA; }
    CUcontext ctx = nullptr;
    if (getCur(&ctx) != CUDA_SUCCESS) { why = "cuCtxGetCurrent failed"; return MOHID_AD_ERR_CUDA; }
    if (!ctx) {
        cudaError_t e = cudaSetDevice(dev);
        if (e != cudaSuccess) { why = std::string("cudaSetDevice: ") + cudaGetErrorString(e); return MOHID_AD_ERR_CUDA; }
        if (getCur(&ctx) != CUDA_SUCCESS || !ctx) { why = "no current CUDA context"; return MOHID_AD_ERR_CUDA; }
    }
    if (getId(ctx, id) != CUDA_SUCCESS) { why = "cuCtxGetId failed"; return MOHID_AD_ERR_CUDA; }
    return MOHID_AD_SUCCESS;
}

int scratch_for_device(int dev, double** out, std::string& why)
{
    if (dev < 0 || dev >= kMaxDevices) { why = "device ordinal out of range"; return MOHID_AD_ERR_CUDA; }
    unsigned long long ctx = 0;
    int code = current_context_id(dev, &ctx, why);
    if (code) return code;
    std::lock_guard<std::mutex> lk(g_mu);
    ScratchSlot& sl = g_scratch[dev];
    if (sl.ctx != ctx) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_row_partials);
        if (e != cudaSuccess) {
            why = std::string("cudaGetSymbolAddress(g_row_partials): ") + cudaGetErrorString(e);
            return MOHID_AD_ERR_CUDA;
        }
        sl.p = static_cast<double*>(p);
        sl.ctx = ctx;
    }
    *out = sl.p;
    return MOHID_AD_SUCCESS;
}

}  // namespace

using namespace mohid_abi;

extern "C" int mohid_ad_mass_f64_noalloc(const T_Size3D* size, const double* PROP, const double* VolumeZ,
                                         const int* WaterPoints3D, double* mass, void* stream, int* stat)
{
    if (!size || !PROP || !VolumeZ || !WaterPoints3D || !mass)
        return fail(MOHID_AD_ERR_NULLPTR, stat, "mohid_ad_mass_f64_noalloc: NULL argument");
    const T_Size3D& s = *size;
    if (s.ILB != 0 || s.JLB != 0 || s.KLB != 0 || s.IUB < 2 || s.JUB < 2 || s.KUB < 2)
        return fail(MOHID_AD_ERR_BOUNDS, stat, "mohid_ad_mass_f64_noalloc: Size must be 0..N+1 in i, j and k");
    const int ni = s.IUB - 1, nj = s.JUB - 1, nk = s.KUB - 1;
    if (nj > kMaxRows)
        return fail(MOHID_AD_ERR_BOUNDS, stat,
                    "mohid_ad_mass_f64_noalloc: JUB - 1 = " + std::to_string(nj) +
                        " work-box rows exceed the fixed scratch of 8192 rows");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(MOHID_AD_ERR_CUDA, stat, cuda_msg("cudaGetDevice", e));
    double* partials = nullptr;
    std::string why;
    int code = scratch_for_device(dev, &partials, why);
    if (code) return fail(code, stat, why);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_row_mass<<<nj, kThreads, 0, st>>>(PROP, VolumeZ, WaterPoints3D, ni, nj, nk, partials);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail(MOHID_AD_ERR_CUDA, stat, cuda_msg("k_row_mass", e));
    k_rows_finish<<<1, 1, 0, st>>>(partials, nj, mass);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail(MOHID_AD_ERR_CUDA, stat, cuda_msg("k_rows_finish", e));
    return ok(stat);
}
