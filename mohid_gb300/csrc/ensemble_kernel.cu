// ensemble_kernel.cu -- many independent domains in one persistent launch.
//
// An ensemble is a set of batched domains (each with its own grid, masks,
// hydrodynamics, DT and tracers) stepped together: one grid of persistent
// CTAs walks a list of (domain, tile) pairs, sorted by the cost of a tile
// (its domain's layer count), so that small and large domains share the GPU
// instead of running one after the other.  Each domain's arguments and tensor
// maps are read from device tables; the tile walk itself is the one of the
// single-domain launch (batched_tile.cuh), so a member steps to the same bits
// in either launch.
#include "batched_tile.cuh"

namespace mohid {
using namespace tile;
namespace {

constexpr int TY = kTY;                            // ensembles walk 32 x 8 tiles
constexpr int NTH = TileGeom<TY>::NTH;

template <int NT, int METHOD, int LIM, bool OBC>
__global__ void __launch_bounds__(NTH, NT <= 2 ? 4 : 3)
ensemble_kernel(const BatchArgs* __restrict__ As, const TmaMaps* __restrict__ Ms,
                const int4* __restrict__ tiles, int ntiles)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(16) BatchArgs sA;         // the current tile's domain
    constexpr int nw = (int)(sizeof(BatchArgs) / sizeof(int));
    static_assert(sizeof(BatchArgs) % sizeof(int) == 0, "BatchArgs copied by words");
    const int tid = threadIdx.y * TX + threadIdx.x;
    uint32_t phase = 0;                            // bit s: parity of stage buffer s
    walk_init<NT, float, float, TY>(smem_raw);
    int cur = -1;
    for (int e = blockIdx.x; e < ntiles; e += gridDim.x) {
        const int4 t = tiles[e];                   // (domain, bx, by, -)
        __syncthreads();                           // every warp is past the previous walk
        if (t.x != cur) {
            const int* src = reinterpret_cast<const int*>(As + t.x);
            for (int w = tid; w < nw; w += NTH) reinterpret_cast<int*>(&sA)[w] = src[w];
            __syncthreads();
            cur = t.x;
        }
        if (!tile_walk<NT, METHOD, LIM, float, float, OBC, TY>(sA, Ms[t.x], t.y, t.z, smem_raw, phase)) return;
    }
}

template <int NT, int METHOD, int LIM, bool OBC>
cudaError_t ens_launch_t(const BatchArgs* As, const TmaMaps* Ms, const int4* tiles, int ntiles, int grid,
                         cudaStream_t s)
{
    const size_t smem = Smem<NT, float, float, TY>::bytes(0);
    auto kern = ensemble_kernel<NT, METHOD, LIM, OBC>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<grid, dim3(TX, TY), smem, s>>>(As, Ms, tiles, ntiles);
    return cudaGetLastError();
}

template <int NT, int METHOD, int LIM>
int ens_slots_t(int device)
{
    const size_t smem = Smem<NT, float, float, TY>::bytes(0);
    auto kern = ensemble_kernel<NT, METHOD, LIM, true>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 0;
    int per = 0, sms = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, NTH, smem) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
    return per * sms;
}

template <int NT, bool OBC>
cudaError_t ens_launch_o(int method, int limiter, const BatchArgs* As, const TmaMaps* Ms, const int4* tiles,
                         int ntiles, int grid, cudaStream_t s)
{
    if (method == 1) return ens_launch_t<NT, 1, 0, OBC>(As, Ms, tiles, ntiles, grid, s);
    switch (limiter) {
    case 1: return ens_launch_t<NT, 4, 1, OBC>(As, Ms, tiles, ntiles, grid, s);
    case 2: return ens_launch_t<NT, 4, 2, OBC>(As, Ms, tiles, ntiles, grid, s);
    case 3: return ens_launch_t<NT, 4, 3, OBC>(As, Ms, tiles, ntiles, grid, s);
    case 4: return ens_launch_t<NT, 4, 4, OBC>(As, Ms, tiles, ntiles, grid, s);
    default: return ens_launch_t<NT, 4, 5, OBC>(As, Ms, tiles, ntiles, grid, s);
    }
}

template <int NT>
cudaError_t ens_launch_n(int method, int limiter, bool open, const BatchArgs* As, const TmaMaps* Ms,
                         const int4* tiles, int ntiles, int grid, cudaStream_t s)
{
    if (open) return ens_launch_o<NT, true>(method, limiter, As, Ms, tiles, ntiles, grid, s);
    return ens_launch_o<NT, false>(method, limiter, As, Ms, tiles, ntiles, grid, s);
}

template <int NT>
int ens_slots_n(int method, int limiter, int device)
{
    if (method == 1) return ens_slots_t<NT, 1, 0>(device);
    switch (limiter) {
    case 1: return ens_slots_t<NT, 4, 1>(device);
    case 2: return ens_slots_t<NT, 4, 2>(device);
    case 3: return ens_slots_t<NT, 4, 3>(device);
    case 4: return ens_slots_t<NT, 4, 4>(device);
    default: return ens_slots_t<NT, 4, 5>(device);
    }
}

}  // namespace

cudaError_t launch_ensemble(const BatchArgs* As, const TmaMaps* Ms, const int4* tiles, int ntiles, int grid,
                            int nt, int method, int limiter, bool open, cudaStream_t s)
{
    if (nt == 4) return ens_launch_n<4>(method, limiter, open, As, Ms, tiles, ntiles, grid, s);
    if (nt == 2) return ens_launch_n<2>(method, limiter, open, As, Ms, tiles, ntiles, grid, s);
    if (nt == 1) return ens_launch_n<1>(method, limiter, open, As, Ms, tiles, ntiles, grid, s);
    return cudaErrorInvalidValue;
}

int ensemble_slots(int nt, int method, int limiter, int device)
{
    if (nt == 4) return ens_slots_n<4>(method, limiter, device);
    if (nt == 2) return ens_slots_n<2>(method, limiter, device);
    if (nt == 1) return ens_slots_n<1>(method, limiter, device);
    return 0;
}

}  // namespace mohid
