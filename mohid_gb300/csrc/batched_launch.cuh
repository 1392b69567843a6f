// batched_launch.cuh -- single-domain launch of the batched FP32 multi-tracer
// transport step (the walk is in batched_tile.cuh): either one CTA per 32 x TY
// tile of the grid, or a persistent grid walking a list of the tiles that hold
// water, costliest (deepest) first -- the column-length-aware schedule for
// z-level domains, whose shallow and land tiles would otherwise cost CTAs.
// Instantiated by batched_inst.cu, once per form, storage and tile height.
#pragma once
#include "batched_tile.cuh"

namespace mohid {
namespace launch_detail {
using namespace tile;

// registers per thread as 32 x 8 tiles have them: 4, 3 or 2 CTAs of 8 warps
// per SM by tracer count, and twice as many CTAs of 4 warps
template <int NT, int TY>
struct MinCtas {
    static constexpr int v8 = NT <= 2 ? 4 : (NT <= 4 ? 3 : 2);
    static constexpr int value = v8 * 8 / TY;
};

template <int NT, int METHOD, int LIM, typename QT, typename KT, int OBC, int TY>
__global__ void __launch_bounds__(TileGeom<TY>::NTH, MinCtas<NT, TY>::value)
batched_kernel(const BatchArgs A, const __grid_constant__ TmaMaps M, const int2* __restrict__ tiles, int ntl)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint32_t phase = 0;                            // bit s: parity of stage buffer s
    walk_init<NT, QT, KT, TY>(smem_raw);
    if (!tiles) {
        tile_walk<NT, METHOD, LIM, QT, KT, OBC, TY>(A, M, blockIdx.x, blockIdx.y, smem_raw, phase);
        return;
    }
    for (int e = blockIdx.x; e < ntl; e += gridDim.x) {
        if (e != (int)blockIdx.x) __syncthreads(); // every warp is past the previous walk
        const int2 t = tiles[e];
        if (!tile_walk<NT, METHOD, LIM, QT, KT, OBC, TY>(A, M, t.x, t.y, smem_raw, phase)) return;
    }
}

template <int NT, int METHOD, int LIM, typename QT, typename KT, int OBC, int TY>
cudaError_t launch_t(const BatchArgs& a, const TmaMaps& m, const int2* tiles, int ntl, cudaStream_t s)
{
    constexpr int NTH = TileGeom<TY>::NTH;
    const size_t smem = Smem<NT, QT, KT, TY>::bytes(a.L.nk, OBC == 2);
    auto kern = batched_kernel<NT, METHOD, LIM, QT, KT, OBC, TY>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (!tiles) {
        dim3 grd((unsigned)((a.L.ni + TX - 1) / TX), (unsigned)((a.L.nj + TY - 1) / TY));
        kern<<<grd, dim3(TX, TY), smem, s>>>(a, m, nullptr, 0);
        return cudaGetLastError();
    }
    // as many CTAs as stay resident (once per instantiation and device)
    static int slots[64] = {};
    int dev = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (!slots[dev]) {
        int per = 0, sms = 0;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, NTH, smem)) != cudaSuccess) return e;
        if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
        slots[dev] = per * sms > 0 ? per * sms : 1;
    }
    const int grid = ntl < slots[dev] ? ntl : slots[dev];
    if (grid < 1) return cudaSuccess;
    kern<<<grid, dim3(TX, TY), smem, s>>>(a, m, tiles, ntl);
    return cudaGetLastError();
}

template <int NT, typename QT, typename KT, int OBC, int TY>
cudaError_t launch_m(const BatchArgs& a, const TmaMaps& m, int method, int limiter, const int2* tiles, int ntl,
                     cudaStream_t s)
{
    if (method == 1) return launch_t<NT, 1, 0, QT, KT, OBC, TY>(a, m, tiles, ntl, s);
    switch (limiter) {
    case 1: return launch_t<NT, 4, 1, QT, KT, OBC, TY>(a, m, tiles, ntl, s);
    case 2: return launch_t<NT, 4, 2, QT, KT, OBC, TY>(a, m, tiles, ntl, s);
    case 3: return launch_t<NT, 4, 3, QT, KT, OBC, TY>(a, m, tiles, ntl, s);
    case 4: return launch_t<NT, 4, 4, QT, KT, OBC, TY>(a, m, tiles, ntl, s);
    default: return launch_t<NT, 4, 5, QT, KT, OBC, TY>(a, m, tiles, ntl, s);
    }
}

// the kernels of one storage (QT transports, KT diffusivities) for every
// tracer group size and scheme
template <int OBC, typename QT, typename KT, int TY>
cudaError_t launch_storage(const BatchArgs& a, const TmaMaps& m, int method, int limiter, const int2* tiles, int ntl,
                           cudaStream_t s)
{
    switch (a.nt) {
    case 10: return launch_m<10, QT, KT, OBC, TY>(a, m, method, limiter, tiles, ntl, s);
    case 8: return launch_m<8, QT, KT, OBC, TY>(a, m, method, limiter, tiles, ntl, s);
    case 4: return launch_m<4, QT, KT, OBC, TY>(a, m, method, limiter, tiles, ntl, s);
    case 2: return launch_m<2, QT, KT, OBC, TY>(a, m, method, limiter, tiles, ntl, s);
    case 1: return launch_m<1, QT, KT, OBC, TY>(a, m, method, limiter, tiles, ntl, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace launch_detail

// One instantiation unit per form (OBC 0: closed boundaries, 1: the
// MassConservation terms compiled in, 2: every open-boundary treatment and
// the discharge terms)
// and storage (0: FP32, 1: FP16 transports, 2: FP16 transports and
// diffusivities) and tile height (8 or 4 rows): batched_inst.cu, compiled
// once per triple in parallel.
template <int OBC, int STORAGE, int TY>
cudaError_t launch_batched_unit(const BatchArgs& a, const TmaMaps& m, int method, int limiter, const int2* tiles,
                                int ntl, cudaStream_t s)
{
    using QT = typename std::conditional<STORAGE >= 1, __half, float>::type;
    using KT = typename std::conditional<STORAGE >= 2, __half, float>::type;
    return launch_detail::launch_storage<OBC, QT, KT, TY>(a, m, method, limiter, tiles, ntl, s);
}
#define MOHID_BATCHED_UNIT(OBC, STORAGE, TY)                                                                 \
    template cudaError_t launch_batched_unit<OBC, STORAGE, TY>(const BatchArgs&, const TmaMaps&, int, int,   \
                                                               const int2*, int, cudaStream_t)
#define MOHID_BATCHED_UNITS_OF(TY)                                                                           \
    extern MOHID_BATCHED_UNIT(0, 0, TY);                                                                     \
    extern MOHID_BATCHED_UNIT(0, 1, TY);                                                                     \
    extern MOHID_BATCHED_UNIT(0, 2, TY);                                                                     \
    extern MOHID_BATCHED_UNIT(1, 0, TY);                                                                     \
    extern MOHID_BATCHED_UNIT(1, 1, TY);                                                                     \
    extern MOHID_BATCHED_UNIT(1, 2, TY);                                                                     \
    extern MOHID_BATCHED_UNIT(2, 0, TY);                                                                     \
    extern MOHID_BATCHED_UNIT(2, 1, TY);                                                                     \
    extern MOHID_BATCHED_UNIT(2, 2, TY)
MOHID_BATCHED_UNITS_OF(8);
MOHID_BATCHED_UNITS_OF(4);

}  // namespace mohid
