// instance.hpp -- internal state shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/mohid_ad.h"
#include "common.cuh"

namespace mohid_abi {

int fail(int code, int* stat, const std::string& msg);
int ok(int* stat);
std::string cuda_msg(const char* what, cudaError_t e);

// test hook (mohid_ad_debug_fail_alloc): when > 0, counts device
// allocations down and fails the one that reaches zero
extern int g_fail_alloc;

template <class T>
struct DevBuf {
    T* p = nullptr;          // the array in use: the own allocation, or a borrowed device array
    T* own = nullptr;
    size_t n = 0;
    cudaError_t alloc(size_t count)
    {
        n = count;
        if (g_fail_alloc > 0 && --g_fail_alloc == 0) { p = own = nullptr; return cudaErrorMemoryAllocation; }
        cudaError_t e = cudaMalloc((void**)&p, sizeof(T) * (count ? count : 1));
        own = e == cudaSuccess ? p : nullptr;
        if (e == cudaSuccess) e = cudaMemset(p, 0, sizeof(T) * (count ? count : 1));
        return e;
    }
    void release()
    {
        if (own) cudaFree(own);
        p = own = nullptr;
    }
    // use the caller's device array in place of the own one (never freed here)
    void borrow(T* x) { p = x; }
    void unborrow() { p = own; }
};

struct Instance {
    int device = 0;
    int ni = 0, nj = 0, nk = 0;
    size_t n2 = 0, n3 = 0;
    cudaStream_t stream = nullptr;
    // static 2-D metrics
    DevBuf<double> DUX, DVY, DZX, DZY;
    DevBuf<int> KFloor, BP2D;
    // boundary columns (2-D offsets, the reference's sweep order) and the rows
    // and columns whose two ends are boundary points (cyclic boundaries)
    DevBuf<int> bcols, cycl;
    int nbcols = 0, nrows = 0, ncyc = 0;
    // per-step hydrodynamics
    DevBuf<double> Qx, Qy, Qz, Vold, V, ViscH, DiffV, AreaU, AreaV, DZZ, DWZ;
    DevBuf<int> OP, LP, WP, CFU, CFV, CFW, SD;
    // face thicknesses DUZ, DVZ of the geometry producer (allocated on first use)
    DevBuf<double> DUZ, DVZ;
    bool hydro = false, hasSD = false;
    unsigned hydroVersion = 0;         // bumped by every change of the per-step hydrodynamics
    unsigned maskVersion = 0;          // bumped by every upload of the 3-D masks
    // per-property staging for the host-pointer entry points
    DevBuf<double> Pin, Pout, Ref;
    // implicit horizontal advection (allocated on first use): the rows of the
    // horizontal system (4 x Size box), the line solver's W, the line solution
    DevBuf<double> sys, Wl, Pmid;
    // Orlanski boundaries (allocated on first use): the field with the
    // radiated exterior values; the caller's PropOld (mohid_ad_set_prop_old)
    DevBuf<double> Pobc;
    double* propOld = nullptr;
    bool propOldDev = false;
    // CellFluxes of the last step (6 x Size box: AdvFluxX/Y/Z, DifFluxX/Y/Z),
    // allocated on first use; fluxLast: the last step computed them
    DevBuf<double> flux;
    bool fluxLast = false;
    // NoFluxU/V/W masks (mohid_ad_set_noflux), used by NoAdvFlux / NoDifFlux
    DevBuf<int> NFU, NFV, NFW;
    bool hasNoFlux = false;
    unsigned nofluxVersion = 0;        // bumped by every mohid_ad_set_noflux
    // discharges (mohid_ad_set_discharges): per-column term lists
    std::vector<int> hKFloor;          // KFloorZ (host copy, Size box 2-D)
    DevBuf<int> dStart;
    DevBuf<mohid::DischTerm> dTerms;
    bool hasDisch = false;
    // host copies of the terms in the same order: term, its Size-box column and
    // its discharge cell n (the index into DischConc); bumped on every change
    std::vector<mohid::DischTerm> hTerms;
    std::vector<int> hTermCol, hTermCell;
    int nDischCells = 0;
    unsigned dischVersion = 0;
    DevBuf<unsigned int> status;
    unsigned int* hstatus = nullptr;   // pinned

    void release();
};

Instance* lookup(const int* id);

// NVTX range around one C-ABI call (a profiler shows each entry point's span;
// without a tool attached the calls do nothing)
struct TraceRange {
    explicit TraceRange(const char* name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange&) = delete;
    TraceRange& operator=(const TraceRange&) = delete;
};

#define CK(call)                                                                  \
    do {                                                                          \
        cudaError_t e_ = (call);                                                  \
        if (e_ != cudaSuccess) return ::mohid_abi::fail(MOHID_AD_ERR_CUDA, stat, ::mohid_abi::cuda_msg(#call, e_)); \
    } while (0)

int status_to_code(unsigned int s, std::string& why);

}  // namespace mohid_abi
