// batched_kernel.cu -- the dispatch of the batched step to its instantiation
// units (batched_inst.cu), the tile-cost kernel of the schedule, and the
// layout queries of the batched form.
#include "batched_launch.cuh"

namespace mohid {
using namespace tile;
namespace {

// tile cost for the schedule: layers walked (KUB - lowest KFloor + 1), 0 without water
template <int TY>
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

// The step kernels' bounded stage wait, on a barrier that nothing completes:
// it gives up after `polls` polls, and the CTA reports MOHID_DEV_TIMEOUT as
// the step's exit path does when a stage never arrives.
__global__ void k_wait_probe(uint32_t polls, unsigned* status)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    const bool ok = mbar_wait_bounded(&bar, 0, polls);
    if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicOr(status, MOHID_DEV_TIMEOUT);
}

template <int NT>
size_t smem_n(bool halfQ, bool halfK, int nk)
{
    if (halfQ && halfK) return Smem<NT, __half, __half, kTY>::bytes(nk);
    if (halfQ) return Smem<NT, __half, float, kTY>::bytes(nk);
    return Smem<NT, float, float, kTY>::bytes(nk);
}

template <int OBC, int STORAGE>
cudaError_t launch_ty(const BatchArgs& a, const TmaMaps& m, int method, int limiter, const int2* tiles, int ntl,
                      int ty, cudaStream_t s)
{
    if (ty == 4) return launch_batched_unit<OBC, STORAGE, 4>(a, m, method, limiter, tiles, ntl, s);
    if (ty == 8) return launch_batched_unit<OBC, STORAGE, 8>(a, m, method, limiter, tiles, ntl, s);
    return cudaErrorInvalidValue;
}

}  // namespace

cudaError_t wait_probe(unsigned polls, unsigned* status, cudaStream_t s)
{
    k_wait_probe<<<1, 32, 0, s>>>(polls, status);
    return cudaGetLastError();
}

// discharges, and open boundaries (reference concentrations set) other than
// MassConservation, take the form with every boundary treatment and the
// discharge terms; MassConservation alone the form with its terms only
cudaError_t launch_batched(const BatchArgs& a, const TmaMaps& m, int method, int limiter, bool halfQ,
                           bool halfK, const int2* tiles, int ntl, int ty, cudaStream_t s)
{
    const int storage = halfQ ? (halfK ? 2 : 1) : 0;
    if (a.dStart || (a.Ref && a.bc != 1)) {
        if (storage == 2) return launch_ty<2, 2>(a, m, method, limiter, tiles, ntl, ty, s);
        if (storage == 1) return launch_ty<2, 1>(a, m, method, limiter, tiles, ntl, ty, s);
        return launch_ty<2, 0>(a, m, method, limiter, tiles, ntl, ty, s);
    }
    if (a.Ref) {
        if (storage == 2) return launch_ty<1, 2>(a, m, method, limiter, tiles, ntl, ty, s);
        if (storage == 1) return launch_ty<1, 1>(a, m, method, limiter, tiles, ntl, ty, s);
        return launch_ty<1, 0>(a, m, method, limiter, tiles, ntl, ty, s);
    }
    if (storage == 2) return launch_ty<0, 2>(a, m, method, limiter, tiles, ntl, ty, s);
    if (storage == 1) return launch_ty<0, 1>(a, m, method, limiter, tiles, ntl, ty, s);
    return launch_ty<0, 0>(a, m, method, limiter, tiles, ntl, ty, s);
}

cudaError_t tile_costs(const uint8_t* cflag, const int* kfloor, const BLayout& L, int tilesX, int ntiles, int ty,
                       int* cost, cudaStream_t s)
{
    if (ty == 4) k_tile_cost<4><<<(ntiles + 127) / 128, 128, 0, s>>>(cflag, kfloor, L, tilesX, ntiles, cost);
    else if (ty == 8) k_tile_cost<8><<<(ntiles + 127) / 128, 128, 0, s>>>(cflag, kfloor, L, tilesX, ntiles, cost);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

size_t batched_smem_bytes(int nt, bool halfQ, bool halfK, int nk)
{
    if (nt == 10) return smem_n<10>(halfQ, halfK, nk);
    if (nt == 8) return smem_n<8>(halfQ, halfK, nk);
    if (nt == 4) return smem_n<4>(halfQ, halfK, nk);
    if (nt == 2) return smem_n<2>(halfQ, halfK, nk);
    return smem_n<1>(halfQ, halfK, nk);
}

// box extents of the tensor maps (elements), for the host-side encoder
void batched_boxes(bool halfQ, bool halfK, int nt, int TY, int box[kNumMaps][4])
{
    const int qyX = halfQ ? Box<__half>::qyX : Box<float>::qyX;
    const int visX = halfK ? Box<__half>::visX : Box<float>::visX;
    const int b[kNumMaps][4] = {{PBX, TY + 4, 1, nt}, {FBX, TY + 1, 1, 1}, {VBX, TY + 2, 1, 1},
                                {visX, TY + 2, 1, 1}, {TX, TY + 1, 1, 1},   {TX, TY + 1, 1, 1},
                                {qyX, TY, 1, 1},      {AVX, TY, 1, 1},      {OWN, TY, 1, 1},
                                {OWN, TY, 1, 1},      {OWN, TY, 1, 1},      {OWN, TY, 1, 1},
                                {OWN, TY, 1, 1}};
    for (int q = 0; q < kNumMaps; ++q)
        for (int d = 0; d < 4; ++d) box[q][d] = b[q][d];
}

}  // namespace mohid
