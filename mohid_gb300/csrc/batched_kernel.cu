// batched_kernel.cu -- single-domain launch of the batched FP32 multi-tracer
// transport step: one CTA per 32 x 8 tile (the walk is in batched_tile.cuh).
#include "batched_tile.cuh"

namespace mohid {
using namespace tile;
namespace {

template <int NT, int METHOD, int LIM, typename QT, typename KT>
__global__ void __launch_bounds__(NTH, NT <= 2 ? 4 : 3)
batched_kernel(const BatchArgs A, const __grid_constant__ TmaMaps M)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint32_t phase = 0;                            // bit s: parity of stage buffer s
    walk_init<NT, QT, KT>(smem_raw);
    tile_walk<NT, METHOD, LIM, QT, KT>(A, M, blockIdx.x, blockIdx.y, smem_raw, phase);
}

template <int NT, int METHOD, int LIM, typename QT, typename KT>
cudaError_t launch_t(const BatchArgs& a, const TmaMaps& m, cudaStream_t s)
{
    const size_t smem = Smem<NT, QT, KT>::bytes(a.L.nk);
    auto kern = batched_kernel<NT, METHOD, LIM, QT, KT>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grd((unsigned)((a.L.ni + TX - 1) / TX), (unsigned)((a.L.nj + TY - 1) / TY));
    kern<<<grd, dim3(TX, TY), smem, s>>>(a, m);
    return cudaGetLastError();
}

template <int NT, typename QT, typename KT>
cudaError_t launch_m(const BatchArgs& a, const TmaMaps& m, int method, int limiter, cudaStream_t s)
{
    if (method == 1) return launch_t<NT, 1, 0, QT, KT>(a, m, s);
    switch (limiter) {
    case 1: return launch_t<NT, 4, 1, QT, KT>(a, m, s);
    case 2: return launch_t<NT, 4, 2, QT, KT>(a, m, s);
    case 3: return launch_t<NT, 4, 3, QT, KT>(a, m, s);
    case 4: return launch_t<NT, 4, 4, QT, KT>(a, m, s);
    default: return launch_t<NT, 4, 5, QT, KT>(a, m, s);
    }
}

template <int NT>
cudaError_t launch_n(const BatchArgs& a, const TmaMaps& m, int method, int limiter, bool halfQ, bool halfK,
                     cudaStream_t s)
{
    if (halfQ && halfK) return launch_m<NT, __half, __half>(a, m, method, limiter, s);
    if (halfQ) return launch_m<NT, __half, float>(a, m, method, limiter, s);
    return launch_m<NT, float, float>(a, m, method, limiter, s);
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
                           bool halfK, cudaStream_t s)
{
    if (a.nt == 4) return launch_n<4>(a, m, method, limiter, halfQ, halfK, s);
    if (a.nt == 2) return launch_n<2>(a, m, method, limiter, halfQ, halfK, s);
    if (a.nt == 1) return launch_n<1>(a, m, method, limiter, halfQ, halfK, s);
    return cudaErrorInvalidValue;
}

size_t batched_smem_bytes(int nt, bool halfQ, bool halfK, int nk)
{
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
