// batched_kernel.cu -- single-domain launch of the batched FP32 multi-tracer
// transport step (the walk is in batched_tile.cuh): either one CTA per 32 x 8
// tile of the grid, or a persistent grid walking a list of the tiles that hold
// water, costliest (deepest) first -- the column-length-aware schedule for
// z-level domains, whose shallow and land tiles would otherwise cost CTAs.
#include "batched_tile.cuh"

namespace mohid {
using namespace tile;
namespace {

template <int NT, int METHOD, int LIM, typename QT, typename KT>
__global__ void __launch_bounds__(NTH, NT <= 2 ? 4 : (NT <= 4 ? 3 : 2))
batched_kernel(const BatchArgs A, const __grid_constant__ TmaMaps M, const int2* __restrict__ tiles, int ntl)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint32_t phase = 0;                            // bit s: parity of stage buffer s
    walk_init<NT, QT, KT>(smem_raw);
    if (!tiles) {
        tile_walk<NT, METHOD, LIM, QT, KT>(A, M, blockIdx.x, blockIdx.y, smem_raw, phase);
        return;
    }
    for (int e = blockIdx.x; e < ntl; e += gridDim.x) {
        if (e != (int)blockIdx.x) __syncthreads(); // every warp is past the previous walk
        const int2 t = tiles[e];
        if (!tile_walk<NT, METHOD, LIM, QT, KT>(A, M, t.x, t.y, smem_raw, phase)) return;
    }
}

template <int NT, int METHOD, int LIM, typename QT, typename KT>
cudaError_t launch_t(const BatchArgs& a, const TmaMaps& m, const int2* tiles, int ntl, cudaStream_t s)
{
    const size_t smem = Smem<NT, QT, KT>::bytes(a.L.nk);
    auto kern = batched_kernel<NT, METHOD, LIM, QT, KT>;
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

template <int NT, typename QT, typename KT>
cudaError_t launch_m(const BatchArgs& a, const TmaMaps& m, int method, int limiter, const int2* tiles, int ntl,
                     cudaStream_t s)
{
    if (method == 1) return launch_t<NT, 1, 0, QT, KT>(a, m, tiles, ntl, s);
    switch (limiter) {
    case 1: return launch_t<NT, 4, 1, QT, KT>(a, m, tiles, ntl, s);
    case 2: return launch_t<NT, 4, 2, QT, KT>(a, m, tiles, ntl, s);
    case 3: return launch_t<NT, 4, 3, QT, KT>(a, m, tiles, ntl, s);
    case 4: return launch_t<NT, 4, 4, QT, KT>(a, m, tiles, ntl, s);
    default: return launch_t<NT, 4, 5, QT, KT>(a, m, tiles, ntl, s);
    }
}

template <int NT>
cudaError_t launch_n(const BatchArgs& a, const TmaMaps& m, int method, int limiter, bool halfQ, bool halfK,
                     const int2* tiles, int ntl, cudaStream_t s)
{
    if (halfQ && halfK) return launch_m<NT, __half, __half>(a, m, method, limiter, tiles, ntl, s);
    if (halfQ) return launch_m<NT, __half, float>(a, m, method, limiter, tiles, ntl, s);
    return launch_m<NT, float, float>(a, m, method, limiter, tiles, ntl, s);
}

// tile cost for the schedule: layers walked (KUB - lowest KFloor + 1), 0 without water
__global__ void k_tile_cost(const uint8_t* cflag, const int* kfloor, BLayout L, int tilesX, int ntiles, int* cost)
{
    const int tile = blockIdx.x * blockDim.x + threadIdx.x;
    if (tile >= ntiles) return;
    const int i0 = 1 + (tile % tilesX) * TX, j0 = 1 + (tile / tilesX) * TY;
    int kmin = L.nk + 1;
    for (int jj = 0; jj < TY; ++jj)
        for (int ii = 0; ii < TX; ++ii) {
            const int i = i0 + ii, j = j0 + jj;
            if (i > L.ni || j > L.nj) continue;
            const long long c = L.at2(i, j);
            if ((cflag[c] & C_SOLVE) && kfloor[c] < kmin) kmin = kfloor[c];
        }
    cost[tile] = kmin <= L.nk ? L.nk - kmin + 1 : 0;
}

template <int NT>
size_t smem_n(bool halfQ, bool halfK, int nk)
{
    if (halfQ && halfK) return Smem<NT, __half, __half>::bytes(nk);
    if (halfQ) return Smem<NT, __half, float>::bytes(nk);
    return Smem<NT, float, float>::bytes(nk);
}

}  // namespace

cudaError_t launch_batched(const BatchArgs& a, const TmaMaps& m, int method, int limiter, bool halfQ,
                           bool halfK, const int2* tiles, int ntl, cudaStream_t s)
{
    if (a.nt == 8) return launch_n<8>(a, m, method, limiter, halfQ, halfK, tiles, ntl, s);
    if (a.nt == 4) return launch_n<4>(a, m, method, limiter, halfQ, halfK, tiles, ntl, s);
    if (a.nt == 2) return launch_n<2>(a, m, method, limiter, halfQ, halfK, tiles, ntl, s);
    if (a.nt == 1) return launch_n<1>(a, m, method, limiter, halfQ, halfK, tiles, ntl, s);
    return cudaErrorInvalidValue;
}

cudaError_t tile_costs(const uint8_t* cflag, const int* kfloor, const BLayout& L, int tilesX, int ntiles, int* cost,
                       cudaStream_t s)
{
    k_tile_cost<<<(ntiles + 127) / 128, 128, 0, s>>>(cflag, kfloor, L, tilesX, ntiles, cost);
    return cudaGetLastError();
}

size_t batched_smem_bytes(int nt, bool halfQ, bool halfK, int nk)
{
    if (nt == 8) return smem_n<8>(halfQ, halfK, nk);
    if (nt == 4) return smem_n<4>(halfQ, halfK, nk);
    if (nt == 2) return smem_n<2>(halfQ, halfK, nk);
    return smem_n<1>(halfQ, halfK, nk);
}

// box extents of the tensor maps (elements), for the host-side encoder
void batched_boxes(bool halfQ, bool halfK, int nt, int box[kNumMaps][4])
{
    const int qyX = halfQ ? Box<__half>::qyX : Box<float>::qyX;
    const int visX = halfK ? Box<__half>::visX : Box<float>::visX;
    const int b[kNumMaps][4] = {{PBX, TY + 4, 1, nt}, {FBX, TY + 1, 1, 1}, {VBX, TY + 2, 1, 1},
                                {visX, TY + 2, 1, 1}, {TX, TY + 1, 1, 1},   {TX, TY + 1, 1, 1},
                                {qyX, TY, 1, 1},      {AVX, TY, 1, 1},      {OWN, TY, 1, 1},
                                {OWN, TY, 1, 1},      {OWN, TY, 1, 1},      {OWN, TY, 1, 1},
                                {OWN, TY, 1, 1},      {OWN, TY, 1, 1},      {OWN, TY, 1, 1}};
    for (int q = 0; q < kNumMaps; ++q)
        for (int d = 0; d < 4; ++d) box[q][d] = b[q][d];
}

}  // namespace mohid
