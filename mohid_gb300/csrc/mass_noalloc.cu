// mass_noalloc.cu -- compensated mass budget that allocates no memory.
//
// Some callers cannot allocate device memory at the point where they need a
// mass budget: a model whose device memory is owned by another allocator (a
// caching allocator that has already reserved the GPU, or a fixed budget
// reserved when the model starts), or code that runs in the middle of a time
// step where an allocation would synchronise the device or fail under memory
// pressure.  For them this file provides the budget with its scratch in a
// file-scope device array: every GPU that loads the library holds these
// 128 KiB (2 x 8192 doubles) until the process exits, and the entry point
// itself calls no allocator.
//
// The sum is the Neumaier-compensated FP64 sum of VolumeZ * PROP over water
// cells of the work box (WaterPoints3D == 1), as the batched form's budget:
// one block per j-row writes a compensated partial (sum, correction) into the
// scratch array, and one thread adds the partials in row order, so the result
// does not depend on scheduling.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/mohid_ad.h"
#include "instance.hpp"

namespace {

constexpr int kMaxRows = 8192;                 // largest JUB (work-box rows) accepted
constexpr int kMaxDevices = 64;

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
    __shared__ double ss[256], sc[256];
    const int j = 1 + blockIdx.x;
    const long long NI = ni + 2, sk = NI * (nj + 2);
    double s = 0.0, c = 0.0;
    const int n = ni * nk;
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
        const int i = 1 + e % ni, k = 1 + e / ni;
        const long long a = i + NI * j + sk * k;
        if (WP[a] == 1) neu_add(s, c, V[a] * P[a]);
    }
    ss[threadIdx.x] = s;
    sc[threadIdx.x] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        double S = 0.0, C = 0.0;
        for (int q = 0; q < (int)blockDim.x; ++q) { neu_add(S, C, ss[q]); C += sc[q]; }
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

// device address of g_row_partials, looked up once per device
std::mutex g_mu;
double* g_scratch[kMaxDevices] = {};

int scratch_for_device(int dev, double** out, std::string& why)
{
    if (dev < 0 || dev >= kMaxDevices) { why = "device ordinal out of range"; return MOHID_AD_ERR_CUDA; }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_row_partials);
        if (e != cudaSuccess) {
            why = std::string("cudaGetSymbolAddress(g_row_partials): ") + cudaGetErrorString(e);
            return MOHID_AD_ERR_CUDA;
        }
        g_scratch[dev] = static_cast<double*>(p);
    }
    *out = g_scratch[dev];
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
                    "mohid_ad_mass_f64_noalloc: JUB = " + std::to_string(nj) +
                        " work-box rows exceed the fixed scratch of 8192 rows");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(MOHID_AD_ERR_CUDA, stat, cuda_msg("cudaGetDevice", e));
    double* partials = nullptr;
    std::string why;
    int code = scratch_for_device(dev, &partials, why);
    if (code) return fail(code, stat, why);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_row_mass<<<nj, 256, 0, st>>>(PROP, VolumeZ, WaterPoints3D, ni, nj, nk, partials);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail(MOHID_AD_ERR_CUDA, stat, cuda_msg("k_row_mass", e));
    k_rows_finish<<<1, 1, 0, st>>>(partials, nj, mass);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail(MOHID_AD_ERR_CUDA, stat, cuda_msg("k_rows_finish", e));
    return ok(stat);
}
