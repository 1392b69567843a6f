// batched.cuh -- layout and arguments of the batched FP32 multi-tracer form.
#pragma once
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace mohid {

// Batched layout of one domain: x = i + kXOff (i = -2..ni+2), y = j + kYOff
// (j = -2..nj+2), z = k (k = 0..nk+1).  kXOff puts the first interior cell of
// every 32-wide tile on a 128-byte boundary.
constexpr int kXOff = 31;
constexpr int kYOff = 2;
constexpr int kTX = 32;   // tile width along i (one warp)
constexpr int kTY = 8;    // tile height along j (warps per CTA): the largest, and the ensembles'
// the tile heights the single-domain kernels are built for (the autotuner's choice)
constexpr int kTileRows[2] = {8, 4};

// cell flag bits; F_NDW / F_NAW: the cell's bottom face carries no diffusion /
// no advection (NoDifFlux / NoAdvFlux with NoFluxW, set by noflux_flags)
constexpr uint8_t F_WP = 1, F_OP = 2, F_CFU = 4, F_CFV = 8, F_CFW = 16, F_LP = 32, F_NDW = 64, F_NAW = 128;
// column flag bits
constexpr uint8_t C_SOLVE = 1, C_OPTOP = 2, C_CFWTOP = 4, C_BP = 8, C_SD = 16;
// face flag bits of a cell's west (U: between j-1 and j) and south (V: between
// i-1 and i) faces: ACT the face is a compute face (ComputeFacesU/V3D), ADV it
// also carries advection (both cells open), TVDP/TVDN the cell upstream of the
// upwind cell is open for a positive/negative transport (not NearBoundary)
constexpr uint8_t FU_ACT = 1, FU_ADV = 2, FU_TVDP = 4, FU_TVDN = 8;
constexpr uint8_t FV_ACT = 16, FV_ADV = 32, FV_TVDP = 64, FV_TVDN = 128;

struct BLayout {
    int ni, nj, nk;
    int px, py;            // pitches in elements
    long long sl;          // layer stride px * py
    long long n3;          // px * py * (nk + 2)
    long long n2;          // px * py
    __host__ __device__ long long at(int i, int j, int k) const
    {
        return (long long)(i + kXOff) + (long long)px * ((long long)(j + kYOff) + (long long)py * k);
    }
    __host__ __device__ long long at2(int i, int j) const
    {
        return (long long)(i + kXOff) + (long long)px * (long long)(j + kYOff);
    }
};

inline BLayout make_layout(int ni, int nj, int nk)
{
    BLayout L;
    L.ni = ni; L.nj = nj; L.nk = nk;
    L.px = ((ni + kXOff + 3 + kTX + 31) / 32) * 32;
    L.py = nj + kYOff + 3 + kTY;
    L.n2 = (long long)L.px * L.py;
    L.sl = L.n2;
    L.n3 = L.n2 * (nk + 2);
    return L;
}

struct BatchArgs {
    BLayout L;
    // shared per-cell fields in the batched layout
    const void *Qx, *Qy, *Qz;           // float or __half (west, south, bottom faces)
    float qsx, qsy, qsz;                // scales for __half storage
    const float *RV;                    // 1/VolumeZ, formed in FP64 (0 where VolumeZ = 0)
    const float *DVR;                   // (VolumeZ - VolumeZOld)/VolumeZ, formed in FP64
    const void *ViscH, *DiffV;          // float or __half
    float ksh, ksv;                     // scales for __half storage
    const float *AreaU, *AreaV, *DZZ;   // DZZ holds 1/DZZ
    const uint8_t* flag;
    const uint8_t* fflag;               // face flag bits (FU_*, FV_*)
    // 2-D: per-face constants [2][py][px] for west (0) and south (1) faces:
    //   x: weight of the cell's own Visc / DZ between the centres
    //   y: weight of the neighbour's Visc / DZ between the centres
    //   z: (du_up + du_dn) / (du_up + du_upup) for Q > 0, w: the same for Q <= 0
    const float4* fc;
    const float* areaCol;               // DUX * DVY
    const int* kfloor;
    const uint8_t* cflag;
    // tracers: contiguous, stride `ts` elements
    const float* Pin;
    float* Pout;
    long long ts;
    int nt;
    // open-boundary references of the boundary columns only (or null): tracer
    // t, boundary column q, layer k at Ref[t * rts + q * rk + k]; refIdx holds
    // q for each column of the layout (-1 away from the boundary)
    const float* Ref;
    const int* refIdx;
    long long rts;
    int rk;
    // discharges (or null; compiled into the open-boundary instantiation): the
    // terms of column c2 of the layout at dTerms[dStart[c2] .. dStart[c2 + 1])
    // (by layer, in the reference's order), tracer t's concentration of term q
    // at dConc[q * ntAll + t]; DWZ (FP64, Size box) for the uniform vertical
    // distribution
    const int* dStart;
    const DischTerm* dTerms;
    const float* dConc;
    const double* DWZ;
    float* W;                           // scratch: THOMASZ W per cell (batched layout)
    float* G;                           // scratch: THOMASZ G of the launch's tracers per cell, nt
                                        // floats per cell (cell c at G + c * nt)
    // mass budget of the fixer (closed domains), or mpart == null: VolumeZ as
    // an FP32 pair hi + lo (batched layout), and per tile and tracer of the
    // batch the sum of VolumeZ * stored value written to
    // mpart[(t0 + t) * ntiles + by * tilesX + bx]
    const float *Vhi, *Vlo;
    double* mpart;
    double* mfix;                       // the batch's fixer state (below)
    // open boundaries under the fixer (else null): the step's boundary mass
    // flux as partials of the obc_flux blocks, obpart[t * nob + blk] = sum of
    // WFOB * DT * value over the block's boundary cells, obpart[ntAll * nob +
    // blk] = sum of WFOB * DT
    double* obpart;
    int nob;
    int tilesX, ntiles, ntAll;          // tiles along i, tiles, tracers of the whole batch
    // scalars
    float DT, schmidtH, coefV, backV, tdec;
    int nullDif, vertical1D, xzflow;
    int bc;                             // BoundaryCondition (with Ref): 1, 2, 5, 7 or 4
    int t0;                             // first tracer of this launch (TMA coordinate)
    unsigned* status;
};

// Tensor maps of one launch: one tiled bulk copy per field and layer.
struct TmaMaps {
    CUtensorMap P;                      // tracers (x, y, z, tracer): box (40, TY+4, 1, NT)
    CUtensorMap F;                      // face flags: box (48, TY+1, 1)
    CUtensorMap V;                      // 1/VolumeZ, f32: box (40, TY+2, 1)
    CUtensorMap Vis;                    // Visc_H: box (40 | 48, TY+2, 1)
    CUtensorMap QX, AU;                 // west faces: box (32, TY+1, 1)
    CUtensorMap QY, AV;                 // south faces: box (36 | 40, TY, 1), (36, TY, 1)
    CUtensorMap Vo;                     // (V - Vold)/V, f32, own cells: box (32, TY, 1)
    CUtensorMap Qz, Dv, Dz, Fn;         // own cells of the layer above / 1/DZZ: box (32, TY, 1)
};

// tiles == null: one CTA per tile of the grid; otherwise a persistent grid over
// the ntl (bx, by) tiles listed.  ty: the tile height (kTileRows); the maps'
// boxes and the argument's tile counts must be those of that height
cudaError_t launch_batched(const BatchArgs& a, const TmaMaps& m, int method, int limiter, bool halfQ,
                           bool halfK, const int2* tiles, int ntl, int ty, cudaStream_t s);
// per tile (by * tilesX + bx) of 32 x ty cells: layers the walk visits, 0 for a tile without water
cudaError_t tile_costs(const uint8_t* cflag, const int* kfloor, const BLayout& L, int tilesX, int ntiles, int ty,
                       int* cost, cudaStream_t s);
size_t batched_smem_bytes(int nt, bool halfQ, bool halfK, int nk);
// ensemble: one persistent grid over the (domain, bx, by, -) tiles of many
// domains with FP32 storage; As/Ms are device tables indexed by domain
// open: some member has reference concentrations (open-boundary instantiation)
cudaError_t launch_ensemble(const BatchArgs* As, const TmaMaps* Ms, const int4* tiles, int ntiles, int grid,
                            int nt, int method, int limiter, bool open, cudaStream_t s);
// test hook: a bounded stage wait that nothing completes (status: MOHID_DEV_TIMEOUT)
cudaError_t wait_probe(unsigned polls, unsigned* status, cudaStream_t s);
// resident CTAs of the ensemble kernel on `device` (0 on error)
int ensemble_slots(int nt, int method, int limiter, int device);
// box extents (elements, x y z w) of the kNumMaps maps in TmaMaps order, for
// tiles of 32 x ty cells
constexpr int kNumMaps = 13;
void batched_boxes(bool halfQ, bool halfK, int nt, int ty, int box[kNumMaps][4]);

// packing (Fortran FP64 Size box <-> batched layout)
// All hydrodynamic fields of one update in one pass: transports and
// diffusivities to FP32 or (halfQ / halfK) to FP16 times inv[0..2] / inv[3..4],
// areas to FP32, 1/DZZ, 1/VolumeZ and (VolumeZ - VolumeZOld)/VolumeZ formed in
// FP64, the cell flag byte (F_*) and the face flag byte (FU_*, FV_*).  dinv
// (device, 5 floats: 1/scale of Qx, Qy, Qz, Visc_H, Diff_V) is read for the
// FP16 fields; may be null for FP32 storage.
cudaError_t pack_fields(const double* Qx, const double* Qy, const double* Qz, const double* V, const double* Vold,
                        const double* Vis, const double* Dif, const double* AU, const double* AV, const double* DZZ,
                        const int* WP, const int* OP, const int* LP, const int* CFU, const int* CFV, const int* CFW,
                        void* oQx, void* oQy, void* oQz, void* oVis, void* oDif, bool halfQ, bool halfK,
                        const float* dinv, float* oAU, float* oAV, float* orDZZ, float* oRV, float* oDVR,
                        float* oVhi, float* oVlo, uint8_t* oflag, uint8_t* offlag, unsigned* moving,
                        const BLayout& L, cudaStream_t s);

// ---- mass fixer.  Per batch a device array
//   mfix[0] = sum of VolumeZ over water cells, mfix[1 + t] = target mass of
//   tracer t (its FP64 mass when loaded plus the boundary flux since),
//   mfix[1 + nt + t] = the constant the stored values are relative to when
//   loaded, mfix[1 + 2 nt + t] = the correction added to that constant since,
//   mfix[1 + 3 nt + t] = the mass that entered through open boundaries since
//   (NaN once the targets are dropped).
// sum of VolumeZ over water cells -> mfix[0] (deterministic)
cudaError_t water_volume(const double* V, const int* WP, const BLayout& L, double* partial, int nblocks,
                         double* mfix, cudaStream_t s);
// tracer t loaded: target = FP64 mass of the Fortran-layout field P, constant = shift, correction = 0
cudaError_t mass_fix_load(const double* P, const double* V, const int* WP, const BLayout& L, double* partial,
                          int nblocks, double shift, int t, int nt, double* mfix, cudaStream_t s);
// new hydrodynamics: *changed = 1 where VolumeZ differs bit for bit from the
// last pack's (Vprev, Fortran layout), and Vprev = Vnew
cudaError_t vol_changed(const double* Vnew, double* Vprev, long long n, unsigned* changed, cudaStream_t s);
// FP16 storage scales of nf FP64 fields on the device (absmax: nf doubles of scratch)
cudaError_t fp16_scales(const double* const* fields, int nf, long long n, double* absmax, float* scale, float* inv,
                        cudaStream_t s);
// after a step: target[t] += the step's boundary flux (obpart != null, nob
// blocks), then, with the step's tile sums (mpart != null),
// correction[t] += (target[t] - mass now) / volume, for every tracer of the
// batch whose target is set
cudaError_t mass_fix_step(const double* mpart, int ntiles, int nt, double* mfix, const double* obpart, int nob,
                          cudaStream_t s);
// targets and boundary fluxes of every tracer dropped (NaN): a step with open
// boundaries ran without the fixer following its boundary flux
cudaError_t mass_fix_drop(double* mfix, int nt, cudaStream_t s);
// Boundary columns (cflag has C_SOLVE and C_BP) in increasing 2-D offset:
// list[0] = count, list[1 .. count] = offsets.  cnt: kObcBlocks ints of scratch.
constexpr int kObcBlocks = 128;
cudaError_t obc_columns(const uint8_t* cflag, const BLayout& L, int* cnt, int* list, cudaStream_t s);
// The step's mass flux through the MassConservation open boundaries, for the
// mass fixer: a covers every tracer of the batch (t0 = 0) with the step's input
// and output buffers; partials to a.obpart (a.nob = kObcBlocks blocks).
cudaError_t obc_flux(const BatchArgs& a, const int* list, bool halfQ, cudaStream_t s);
// CellFluxes of one tracer's last step (batched_flux.cu): the advective (adv)
// or diffusive face fluxes through each cell's west, south and bottom face,
// from the field before the step (Pold, explicit horizontal terms) and after it
// (Pnew, implicit vertical terms), into out[0 .. 3 n3) over the Size box;
// stored values + shift + *corr are the absolute values (corr may be null)
cudaError_t cell_fluxes_batched(const BatchArgs& a, const float* Pold, const float* Pnew, double shift,
                                const double* corr, bool adv, double* out, long long n3, int method, int limiter,
                                bool halfQ, bool halfK, cudaStream_t s);
// the same for `nb` batches from their argument records (device): mpart and
// obpart of each record select what runs for that batch
cudaError_t mass_fix_step_many(const BatchArgs* As, int nb, int ntmax, cudaStream_t s);
// pack_fields, vol_changed, water_volume and (DT > 0) the constant-preservation
// check of continuity_residual in one pass, into *cont (m: the largest
// magnitude among each cell's terms in place of their sum); masks: the flag
// bytes are formed from the masks (they changed), else the stored ones are
// read.  vpart: 2 * nvblocks doubles of scratch (nvblocks <= 16384).
cudaError_t pack_state(const double* Qx, const double* Qy, const double* Qz, const double* V, const double* Vold,
                       const double* Vis, const double* Dif, const double* AU, const double* AV, const double* DZZ,
                       const int* WP, const int* OP, const int* LP, const int* CFU, const int* CFV, const int* CFW,
                       const int* BP2D, bool masks, void* oQx, void* oQy, void* oQz, void* oVis, void* oDif,
                       bool halfQ, bool halfK, const float* dinv, float* oAU, float* oAV, float* orDZZ, float* oRV,
                       float* oDVR, float* oVhi, float* oVlo, uint8_t* oflag, uint8_t* offlag, unsigned* moving,
                       double* Vprev, unsigned* vchanged, double* vpart, int nvblocks, double* mfix, double DT,
                       double tol, double* cont, const BLayout& L, cudaStream_t s);
cudaError_t pack_columns(const double* DUX, const double* DVY, const double* DZX, const double* DZY,
                         const int* KFloor, const int* BP2D, const int* WP, const int* OP,
                         const int* CFW, const int* SD, float4* fc, float* areaCol,
                         int* kfloor, uint8_t* cflag, const BLayout& L, cudaStream_t s);
// Tracers are held as the anomaly P - shift on water cells (shift: a per-tracer
// constant, the mean over water cells): when the step preserves constants it is
// shift-equivariant, and the FP32 rounding then scales with the anomaly rather
// than with the absolute value.
cudaError_t pack_tracer(const double* src, float* dstA, float* dstB, const int* KFloor,
                        const int* WP, double shift, const BLayout& L, cudaStream_t s);
// shift: the stored values' constant; corr (device, may be null): a correction added to it
cudaError_t unpack_tracer(const float* src, double* dst, const double* orig, const int* WP,
                          const int* KFloor, double shift, const double* corr, const BLayout& L, cudaStream_t s);
// open-boundary references: column q of `cols` (Size-box 2-D offsets i + (ni+2) j)
// at layer k to dst[q * (nk+2) + k], relative to the tracer's constant on water
// cells; back to absolute values; and each boundary column's q in the layout
cudaError_t pack_ref(const double* src, const int* WP, const int* cols, int ncols, int ni, int nj, int nk,
                     double shift, float* dst, cudaStream_t s);
cudaError_t unshift_ref(float* R, const int* WP, const int* cols, int ncols, int ni, int nj, int nk, double shift,
                        cudaStream_t s);
cudaError_t ref_index(const int* cols, int ncols, int ni, const BLayout& L, int* idx, cudaStream_t s);
// ImposeNullGradient (AD:1926-1987) on nt batched FP32 tracers (stride ts):
// at each layer the boundary columns `cols` (Size-box 2-D offsets, the
// reference's order) take in turn the mean of their neighbours across compute
// faces (the cell flags' F_CFU / F_CFV); KFloor over the Size box
cudaError_t null_gradient_batched(float* P, long long ts, int nt, const uint8_t* flag, const int* cols, int ncols,
                                  const int* KFloor, const BLayout& L, cudaStream_t s);
// Prop_CyclicBoundary (AD:2121-2224) on nt batched FP32 tracers after the
// solve: the boundary columns `cols` take their compact references (Ref, row
// q of column q, rk values, tracer stride rts; less corr[t]), then the rows and
// columns whose two ends are boundary points (BP: BoundaryPoints2D, Size box)
// copy the interior values next to the opposite end from KFloor up
cudaError_t cyclic_batched(float* P, long long ts, int nt, const float* Ref, long long rts, int rk,
                           const double* corr, const int* cols, int ncols, const int* BP, const int* KFloor,
                           const BLayout& L, cudaStream_t s);
// NoAdvFlux / NoDifFlux with the NoFluxU/V/W masks (Size box, may be null when
// both are off) folded into the packed cell and face flags; both off restores
// the unmasked flags.  OP, CFU, CFV, KF: the instance's masks and KFloorZ
cudaError_t noflux_flags(const int* OP, const int* CFU, const int* CFV, const int* NFU, const int* NFV,
                         const int* NFW, const int* KF, bool noAdv, bool noDif, uint8_t* flag, uint8_t* fflag,
                         const BLayout& L, cudaStream_t s);
cudaError_t pack_shift_f32(const double* src, float* dst, const int* WP, double shift, const BLayout& L,
                           cudaStream_t s);
cudaError_t water_mean(const double* src, const int* WP, const BLayout& L, double* partial, int nblocks,
                       double* out, cudaStream_t s);
// *out = max(0, max over open non-boundary water cells of |R| - tol * max |term|),
// R the cell's water budget, and on the top cell of open boundary columns R =
// the surface flux (the step maps constants onto themselves when *out == 0).
// BP2D null: no open-boundary treatment, boundary columns are checked like
// the others (pack_state likewise)
cudaError_t continuity_residual(const double* Qx, const double* Qy, const double* Qz, const double* V,
                                const double* Vold, const int* OP, const int* CFU, const int* CFV,
                                const int* CFW, const int* BP2D, double DT, double tol, const BLayout& L,
                                double* out, cudaStream_t s);
cudaError_t unshift(float* P, const uint8_t* flag, double shift, long long n, cudaStream_t s);
cudaError_t absmax_f64(const double* src, long long n, double* out, cudaStream_t s);
// V: VolumeZ in the Fortran Size-box layout (FP64)
cudaError_t mass_batched(const float* P, const double* V, const uint8_t* flag, double shift, const double* corr,
                         const BLayout& L, double* partial, int nblocks, cudaStream_t s);
cudaError_t mass_finish(const double* partial, int nblocks, double* out, cudaStream_t s);

}  // namespace mohid
