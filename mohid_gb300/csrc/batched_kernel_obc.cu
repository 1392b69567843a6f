// batched_kernel_obc.cu -- open-boundary instantiation of the batched step
// (batched_launch.cuh): MassConservation boundary terms compiled in.
#include "batched_launch.cuh"

namespace mohid {

cudaError_t launch_batched_open(const BatchArgs& a, const TmaMaps& m, int method, int limiter, bool halfQ,
                                bool halfK, const int2* tiles, int ntl, cudaStream_t s)
{
    return launch_detail::launch_batched_form<true>(a, m, method, limiter, halfQ, halfK, tiles, ntl, s);
}

}  // namespace mohid
