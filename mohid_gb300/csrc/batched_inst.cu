// batched_inst.cu -- one instantiation unit of the batched step kernels
// (batched_launch.cuh): the form MOHID_INST_OBC (0: closed, 1: with the
// MassConservation terms, 2: with every open-boundary treatment and the
// discharge terms), the storage MOHID_INST_STORAGE (0: FP32, 1: FP16
// transports, 2: FP16 transports and diffusivities) and the tile height
// MOHID_INST_TY (8 or 4 rows), for every tracer group size and scheme.  The
// build compiles this file once per triple, in parallel.
#include "batched_launch.cuh"

#if !defined(MOHID_INST_OBC) || !defined(MOHID_INST_STORAGE) || !defined(MOHID_INST_TY)
#error "compile with -DMOHID_INST_OBC=0|1|2 -DMOHID_INST_STORAGE=0|1|2 -DMOHID_INST_TY=8|4"
#endif

namespace mohid {
MOHID_BATCHED_UNIT(MOHID_INST_OBC, MOHID_INST_STORAGE, MOHID_INST_TY);
}  // namespace mohid
