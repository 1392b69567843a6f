// batched_abi.cpp -- C-ABI of the batched FP32 multi-tracer form (include/mohid_ad.h).
//
// A batch shares the grid and hydrodynamics of a plain instance (the same
// arguments AdvectionDiffusion receives per property) and transports `nt`
// tracers per call, device-resident, with one option set for all of them
// (one MOHID property group).  The hydrodynamics are repacked on the device
// into the batched layout (FP32 or scaled FP16 transports, FP64 volumes,
// 1-byte masks); tracers are held in FP32 ping-pong buffers.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/mohid_ad.h"
#include "batched.cuh"
#include "instance.hpp"

namespace mohid_abi {
namespace {

struct Batch {
    int plain = 0;
    Instance* in = nullptr;
    int nt = 0;
    int storage = 0;                     // 0 FP32, 1 FP16 transports, 2 FP16 transports + diffusivities
    mohid::BLayout L{};
    DevBuf<float> Qx32, Qy32, Qz32, Vis32, Dif32;
    DevBuf<__half> Qx16, Qy16, Qz16, Vis16, Dif16;
    float qsx = 1, qsy = 1, qsz = 1, ksh = 1, ksv = 1;
    DevBuf<float> RV, DVR;               // 1/V and (V - Vold)/V, both formed in FP64
    DevBuf<float> AreaU, AreaV, DZZ;
    DevBuf<uint8_t> flag, fflag, cflag;
    DevBuf<float4> fc;
    DevBuf<float> areaCol;
    DevBuf<int> kfloor;
    DevBuf<float> PA, PB, Ref;           // tracers (ping-pong); references of the boundary columns
    DevBuf<int> refIdx;                  // per column of the layout: its row in Ref, or -1
    // discharges of the plain instance in the batched layout, with each
    // tracer's concentrations (mohid_ad_batched_set_discharge_conc)
    DevBuf<int> dStart;
    DevBuf<mohid::DischTerm> dTerms;
    DevBuf<float> dConc;
    std::vector<std::vector<double>> hConc;   // per tracer: DischConc of the discharge cells
    unsigned dischVersion = ~0u;         // the instance's discharges the lists hold
    bool dischDirty = true;              // concentrations changed since the upload
    bool dischOn = false;                // the steps apply discharges
    unsigned dischUploads = 0;           // bumped by every upload of the lists
    DevBuf<float> Wsc, Gsc;              // THOMASZ W and G per cell, scratch of the step kernel
    // mass fixer (static volumes): VolumeZ as an FP32 pair, the fixer state
    // (volume, targets, constants, corrections, boundary fluxes), per-tile
    // sums; with open boundaries the boundary columns and the per-block
    // boundary fluxes of a step
    DevBuf<float> Vhi, Vlo;
    DevBuf<double> mfix, mpart, obpart;
    DevBuf<int> obcol, obcnt;
    DevBuf<double> Vprev;                // VolumeZ of the last pack (Fortran layout)
    DevBuf<unsigned> moving;
    bool massFix = true;                 // requested (mohid_ad_batched_set_mass_fix)
    bool bcFix = true;                   // the step's boundary condition lets the fixer run (bc_fixable)
    bool staticVol = false;              // the packed hydrodynamics have VolumeZ == VolumeZOld
    bool packedOnce = false;
    unsigned packedMask = 0;             // mask version of the last completed pack
    unsigned packingMask = 0;            // ... and of the pack in flight
    bool packingMasks = true;            // the pack in flight formed flags and schedule from the masks
    DevBuf<double> vpart;                // per-block water-volume sums of the pack
    bool fixDirty = false;               // the device constants / corrections differ from `shift`
    // launch schedule: one CTA per tile, or a persistent grid over the tiles
    // holding water, costliest first; tracers per launch; the tile height
    // (kTileRows[th]); chosen by timing.  Tile counts, lists, costs and
    // tensor maps are kept for each height (index h of kTileRows)
    int tilesX = 0, ntiles[2] = {0, 0};
    DevBuf<int2> tl[2];
    DevBuf<int> tcost[2];
    int ntl[2] = {0, 0};
    int sched = 0;                       // 0 grid, 1 tile list
    int split = 4;                       // largest tracer group per launch: 10, 8, 4 or 2
    int th = 0;                          // tile height in use: kTileRows[th] rows
    int sumsTh = 0;                      // the height the fixer's per-tile sums are laid out for
    bool tuned = false;
    int graphSched = -1, graphSplit = -1, graphTh = -1;
    int graphFix = -1;                   // fixer / open-boundary launches the graph holds
    bool graphLast = false;              // the graph ends with the call's last step
    unsigned graphPack = ~0u;            // packed hydrodynamics the graph's arguments hold
    unsigned graphDisch = ~0u;           // discharge upload the graph's arguments hold (dischUploads)
                                         // (FP16 scales, tile count)
    // asynchronous repack of a new hydrodynamic state (on the instance's
    // stream) and tracer loads (on their own stream, with their own scratch),
    // so that the two overlap; the host-side results of the repack are read
    // when a step needs them (pack_finalize)
    cudaStream_t cs = nullptr;           // tracer loads
    cudaEvent_t packEv = nullptr;
    bool packPending = false;
    unsigned packingVersion = ~0u;
    struct PackHost {
        unsigned moving, vchanged;
        float scale[5];
        double cont;                     // continuity excess for contDT, or -1 when not computed
        double contDT;
    };
    PackHost* hp = nullptr;              // pinned
    int* hcost[2] = {nullptr, nullptr};  // pinned, per tile of each height
    DevBuf<float> dscale, dinv;
    DevBuf<unsigned> vchanged;
    DevBuf<double> tpartial, tscratch;   // scratch of the tracer loads
    std::vector<unsigned> targetVersion; // hydro version each tracer's mass target was taken at
    double preCont = -1.0, preContDT = -1.0;
    unsigned preContVersion = ~0u;
    // the repack's check treated the boundary columns as open boundaries
    // (the batch had references) -- of the last completed pack, of the one in flight
    bool preContRef = false, packingRef = false;
    std::vector<double> shift;           // per tracer: water cells hold P - shift
    std::vector<double> refShift;        // shift each stored reference was packed with
    // anomaly storage is exact only when the step preserves constants; this
    // is re-checked when the hydrodynamics, DT or the flux-set flags change
    unsigned checkedVersion = ~0u;
    double checkedDT = -1.0;
    int checkedFlags = -1;
    bool shiftOk = true;
    // NoAdvFlux (1) / NoDifFlux (2) folded into the packed flags, and the
    // instance's NoFlux masks they were formed from (noflux_flags)
    int nfApplied = 0;
    unsigned nfVersion = ~0u;
    // CellFluxes: the last step call asked for them (with these options) and
    // the ping-pong buffers still hold that step's old and new fields
    bool fluxLast = false;
    mohid_ad_params fluxParams{};
    DevBuf<double> fluxOut;              // 3 Size-box arrays, allocated on first use
    bool hasRef = false;
    bool cur = false;                    // false: PA holds the current state
    int ensemble = 0;                    // id of the ensemble stepping this batch, or 0
    bool packed = false;
    unsigned packedVersion = ~0u;
    DevBuf<double> partial, scratch, stage;
    double* hmass = nullptr;             // pinned
    mohid::TmaMaps maps[2]{};            // shared-field maps per tile height (valid after a pack)
    CUtensorMap mapP[2][2][5];           // tracer maps: tile height x input buffer (A/B) x group size
                                         // (1, 2, 4, 8, 10)
    bool mapsOk = false;
    cudaGraphExec_t graph = nullptr;
    int graphSteps = 0;
    bool graphCur = false;
    mohid_ad_params graphParams{};

    void release()
    {
        DevBuf<float>* f[] = {&Qx32, &Qy32, &Qz32, &Vis32, &Dif32, &AreaU, &AreaV, &DZZ,
                              &areaCol, &PA, &PB, &Ref, &Wsc, &Gsc, &Vhi, &Vlo};
        for (auto* b : f) b->release();
        DevBuf<__half>* h[] = {&Qx16, &Qy16, &Qz16, &Vis16, &Dif16};
        for (auto* b : h) b->release();
        RV.release(); DVR.release(); flag.release(); fflag.release(); cflag.release(); fc.release();
        kfloor.release();
        partial.release(); scratch.release(); stage.release(); refIdx.release();
        dStart.release(); dTerms.release(); dConc.release();
        mfix.release(); mpart.release(); moving.release(); Vprev.release(); vpart.release(); fluxOut.release();
        obpart.release(); obcol.release(); obcnt.release();
        for (int h = 0; h < 2; ++h) { tl[h].release(); tcost[h].release(); }
        dscale.release(); dinv.release(); vchanged.release(); tpartial.release(); tscratch.release();
        if (hp) cudaFreeHost(hp);
        for (int h = 0; h < 2; ++h) {
            if (hcost[h]) cudaFreeHost(hcost[h]);
            hcost[h] = nullptr;
        }
        hp = nullptr;
        if (cs) cudaStreamDestroy(cs);
        if (packEv) cudaEventDestroy(packEv);
        cs = nullptr;
        packEv = nullptr;
        if (hmass) cudaFreeHost(hmass);
        hmass = nullptr;
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
    }
    float* cur_in() { return cur ? PB.p : PA.p; }
    float* cur_out() { return cur ? PA.p : PB.p; }
};

std::mutex g_bmu;
std::map<int, Batch*> g_batch;
int g_next_bid = 1;
constexpr int kMassBlocks = 1024;
constexpr int kPackBlocks = 8192;            // blocks of the per-cell repack pass

Batch* blookup(const int* bid)
{
    if (!bid) return nullptr;
    std::lock_guard<std::mutex> lk(g_bmu);
    auto it = g_batch.find(*bid);
    return it == g_batch.end() ? nullptr : it->second;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point
PFN_cuTensorMapEncodeTiled_v12000 encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// Tiled map over a batched-layout array (x = px, y = py, z = nk+2[, w = nt]).
bool encode_map(CUtensorMap* m, CUtensorMapDataType dt, int elt, const void* base, const mohid::BLayout& L,
                int nw, const int box[4], int rank = 3)
{
    auto enc = encoder();
    if (!enc) return false;
    cuuint64_t dims[4] = {(cuuint64_t)L.px, (cuuint64_t)L.py, (cuuint64_t)(L.nk + 2), (cuuint64_t)nw};
    cuuint64_t strides[3] = {(cuuint64_t)L.px * elt, (cuuint64_t)L.px * L.py * elt,
                             (cuuint64_t)L.px * L.py * (L.nk + 2) * elt};
    cuuint32_t bx[4] = {(cuuint32_t)box[0], (cuuint32_t)box[1], (cuuint32_t)box[2], (cuuint32_t)box[3]};
    cuuint32_t es[4] = {1, 1, 1, 1};
    CUresult r = enc(m, dt, (cuuint32_t)rank, const_cast<void*>(base), dims, strides, bx, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

int check_batched_params(const mohid_ad_params* p, bool hasRef, std::string& why, bool ensemble = false)
{
    if (!p) { why = "params is NULL"; return MOHID_AD_ERR_NULLPTR; }
    if (!(p->DTProp > 0.0) || !std::isfinite(p->DTProp)) { why = "DTProp must be > 0"; return MOHID_AD_ERR_OPTION; }
    if (p->AdvMethodH != MOHID_UPWIND_ORDER1 && p->AdvMethodH != MOHID_P2_TVD) {
        why = "batched form: AdvMethodH must be UpwindOrder1 or P2_TVD (use the plain form)"; return MOHID_AD_ERR_UNSUPPORTED;
    }
    if (p->AdvMethodH == MOHID_P2_TVD && !p->Upwind2H) { why = "P2_TVD needs Upwind2H near boundaries"; return MOHID_AD_ERR_OPTION; }
    if (p->AdvMethodH == MOHID_P2_TVD && (p->TVDLimitationH < 1 || p->TVDLimitationH > 5)) { why = "TVDLimitationH must be 1..5"; return MOHID_AD_ERR_OPTION; }
    if (p->AdvMethodV != MOHID_UPWIND_ORDER1 || p->ImpExp_AdvV != 1.0) {
        why = "batched form: vertical advection must be implicit UpwindOrder1"; return MOHID_AD_ERR_UNSUPPORTED;
    }
    if (p->ImpExp_DifV != 1.0) { why = "batched form: vertical diffusion must be implicit"; return MOHID_AD_ERR_UNSUPPORTED; }
    if (p->ImpExp_DifH != 0.0) { why = "horizontal diffusion must be explicit (reference ERR02)"; return MOHID_AD_ERR_OPTION; }
    if (p->ImpExp_AdvXX != 0.0 || p->ImpExp_AdvYY != 0.0) { why = "implicit horizontal advection not implemented"; return MOHID_AD_ERR_UNSUPPORTED; }
    if (p->Docycle_method != 1) { why = "batched form follows Docycle_method 1"; return MOHID_AD_ERR_UNSUPPORTED; }
    if (p->AdvectionNudging) { why = "option not implemented"; return MOHID_AD_ERR_UNSUPPORTED; }
    if (p->CellFluxes && ensemble) { why = "ensembles: CellFluxes (step the batch alone)"; return MOHID_AD_ERR_UNSUPPORTED; }
    if ((p->NoAdvFlux || p->NoDifFlux) && (hasRef || ensemble)) {
        why = "batched form: NoFlux masks with open-boundary references or in ensembles (use the plain form)";
        return MOHID_AD_ERR_UNSUPPORTED;
    }
    const int bc = p->BoundaryCondition;
    if (hasRef) {
        if (bc != 1 && bc != 2 && bc != 4 && bc != 5 && bc != 6 && bc != 7 && bc != 8) {
            why = "invalid BoundaryCondition (reference Set_Internal_State ERR01)"; return MOHID_AD_ERR_OPTION;
        }
        if (bc == MOHID_BC_ORLANSKI) {
            why = "batched form: Orlanski boundaries (use the plain form)"; return MOHID_AD_ERR_UNSUPPORTED;
        }
        if (ensemble && bc != MOHID_BC_MASS_CONSERVATION) {
            why = "ensembles: closed or MassConservation open boundaries"; return MOHID_AD_ERR_UNSUPPORTED;
        }
    } else if (bc == MOHID_BC_CYCLIC) {
        why = "cyclic boundaries read ReferenceProp (reference Prop_CyclicBoundary)"; return MOHID_AD_ERR_OPTION;
    } else if (ensemble && bc == MOHID_BC_NULL_GRADIENT) {
        why = "ensembles: NullGradient boundaries (use a batch per domain)"; return MOHID_AD_ERR_UNSUPPORTED;
    }
    return MOHID_AD_SUCCESS;
}

// relative continuity residual below which the step maps constants onto themselves
constexpr double kContinuityTol = 1e-9;

// the mass fixer runs where the step maps constants onto themselves (anomaly
// storage valid) and the volumes do not move; with open boundaries its
// targets follow the boundary flux of every step
bool fix_active(const Batch* b)
{
    return b->massFix && b->shiftOk && b->staticVol && b->bcFix;
}

// the step's budget closes through the boundary flux the fixer follows:
// closed domains (NullGradient excepted, whose sweep after the solve sets
// the boundary cells) and MassConservation open boundaries
bool bc_fixable(const Batch* b, const mohid_ad_params* p)
{
    const int bc = p->BoundaryCondition;
    if (b->dischOn) return false;                // discharges add and remove mass
    return b->hasRef ? bc == MOHID_BC_MASS_CONSERVATION : bc != MOHID_BC_NULL_GRADIENT;
}

// The plain instance's discharges in the batched layout with every tracer's
// concentrations; dischOn says whether the steps apply them.  Terms keep the
// instance's order (by column, j outer and i inner, then layer and the
// reference's order), which is also the batched layout's column order.
int ensure_discharges(Batch* b, int* stat)
{
    Instance* in = b->in;
    b->dischOn = in->hasDisch;
    if (!in->hasDisch) return ok(stat);
    for (int t = 0; t < b->nt; ++t)
        if (t >= (int)b->hConc.size() || (int)b->hConc[t].size() != in->nDischCells)
            return fail(MOHID_AD_ERR_OPTION, stat,
                        "set the discharge concentrations of every tracer (mohid_ad_batched_set_discharge_conc)");
    if (b->dischVersion == in->dischVersion && !b->dischDirty) return ok(stat);
    const size_t nq = in->hTerms.size();
    const int sj = in->ni + 2;
    std::vector<int> start((size_t)b->L.n2 + 1, 0);
    for (size_t q = 0; q < nq; ++q) {
        const int c = in->hTermCol[q];
        ++start[(size_t)b->L.at2(c % sj, c / sj) + 1];
    }
    for (long long c = 0; c < b->L.n2; ++c) start[(size_t)c + 1] += start[(size_t)c];
    std::vector<float> conc(nq * (size_t)b->nt);
    for (size_t q = 0; q < nq; ++q)
        for (int t = 0; t < b->nt; ++t) conc[q * (size_t)b->nt + t] = (float)b->hConc[t][(size_t)in->hTermCell[q]];
    CK(cudaStreamSynchronize(in->stream));      // no step still reads the old lists
    auto bad = [&](cudaError_t e) { return fail(MOHID_AD_ERR_ALLOC, stat, cuda_msg("cudaMalloc", e)); };
    cudaError_t e;
    if (!b->dStart.p && (e = b->dStart.alloc((size_t)b->L.n2 + 1)) != cudaSuccess) return bad(e);
    b->dTerms.release(); b->dConc.release();
    if ((e = b->dTerms.alloc(std::max<size_t>(1, nq))) != cudaSuccess) return bad(e);
    if ((e = b->dConc.alloc(std::max<size_t>(1, conc.size()))) != cudaSuccess) return bad(e);
    CK(cudaMemcpy(b->dStart.p, start.data(), sizeof(int) * start.size(), cudaMemcpyHostToDevice));
    if (nq) {
        CK(cudaMemcpy(b->dTerms.p, in->hTerms.data(), sizeof(mohid::DischTerm) * nq, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(b->dConc.p, conc.data(), sizeof(float) * conc.size(), cudaMemcpyHostToDevice));
    }
    b->dischVersion = in->dischVersion;
    b->dischDirty = false;
    ++b->dischUploads;
    return ok(stat);
}

// which of the fixer's launches a step makes (fixer, boundary flux, target drop)
int fix_key(const Batch* b)
{
    return (fix_active(b) ? 1 : 0) | (b->hasRef ? 2 : 0);
}

// Fold the fixer's corrections into the host-side constants (shift[t] = constant
// + correction, correction = 0) and forget the targets: the field stays exactly
// what it was, the fixer stops until the tracers are reloaded.
cudaError_t fix_fold(Batch* b)
{
    if (!b->fixDirty) return cudaSuccess;
    const int nt = b->nt;
    std::vector<double> mf(1 + 4 * nt);
    cudaError_t e = cudaStreamSynchronize(b->in->stream);
    if (e == cudaSuccess) e = cudaMemcpy(mf.data(), b->mfix.p, sizeof(double) * mf.size(), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return e;
    for (int t = 0; t < nt; ++t) {
        b->shift[t] = mf[1 + nt + t] + mf[1 + 2 * nt + t];
        mf[1 + t] = std::nan("");
        mf[1 + nt + t] = b->shift[t];
        mf[1 + 2 * nt + t] = 0.0;
        mf[1 + 3 * nt + t] = std::nan("");
    }
    e = cudaMemcpy(b->mfix.p, mf.data(), sizeof(double) * mf.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) b->fixDirty = false;
    return e;
}

// Enqueue the repack of the instance's current hydrodynamics on the instance's
// stream, without waiting for it: FP16 scales (device side), the fused field
// pack, the water volume of the mass fixer, the per-column data, the tile
// costs of the schedule, the volume-change flag and (for the last DT a step
// used) the continuity check.  pack_finalize collects the results.
int pack_enqueue(Batch* b, int* stat)
{
    Instance* in = b->in;
    if (!in->hydro) return fail(MOHID_AD_ERR_OPTION, stat, "the plain instance has no hydrodynamics set");
    cudaStream_t s = in->stream;
    const mohid::BLayout& L = b->L;
    const bool hq = b->storage >= 1, hk = b->storage >= 2;
    if (hq || hk) {
        const double* f[5] = {in->Qx.p, in->Qy.p, in->Qz.p, in->ViscH.p, in->DiffV.p};
        CK(mohid::fp16_scales(f, 5, (long long)in->n3, b->scratch.p, b->dscale.p, b->dinv.p, s));
        CK(cudaMemcpyAsync(b->hp->scale, b->dscale.p, 5 * sizeof(float), cudaMemcpyDeviceToHost, s));
    }
    // the per-cell pass (fields, flag bytes when the masks changed, volume
    // change, water volume, and the constant-preservation check for the DT of
    // the last step); the per-column data and the tile schedule only when the
    // masks changed
    const bool masks = !b->packedOnce || b->packedMask != in->maskVersion;
    const double cdt = (b->checkedDT > 0.0 && (b->checkedFlags & 3) == 0) ? b->checkedDT : 0.0;
    CK(mohid::pack_state(in->Qx.p, in->Qy.p, in->Qz.p, in->V.p, in->Vold.p, in->ViscH.p, in->DiffV.p,
                         in->AreaU.p, in->AreaV.p, in->DZZ.p, in->WP.p, in->OP.p, in->LP.p, in->CFU.p,
                         in->CFV.p, in->CFW.p, b->hasRef ? in->BP2D.p : nullptr, masks,
                         hq ? (void*)b->Qx16.p : (void*)b->Qx32.p, hq ? (void*)b->Qy16.p : (void*)b->Qy32.p,
                         hq ? (void*)b->Qz16.p : (void*)b->Qz32.p, hk ? (void*)b->Vis16.p : (void*)b->Vis32.p,
                         hk ? (void*)b->Dif16.p : (void*)b->Dif32.p, hq, hk, (hq || hk) ? b->dinv.p : nullptr,
                         b->AreaU.p, b->AreaV.p, b->DZZ.p, b->RV.p, b->DVR.p, b->Vhi.p, b->Vlo.p, b->flag.p,
                         b->fflag.p, b->moving.p, b->Vprev.p, b->vchanged.p, b->vpart.p, kPackBlocks, b->mfix.p,
                         cdt, kContinuityTol, b->scratch.p + 5, L, s));
    if (masks) {
        CK(mohid::pack_columns(in->DUX.p, in->DVY.p, in->DZX.p, in->DZY.p, in->KFloor.p, in->BP2D.p,
                               in->WP.p, in->OP.p, in->CFW.p, in->hasSD ? in->SD.p : nullptr,
                               b->fc.p, b->areaCol.p, b->kfloor.p, b->cflag.p, L, s));
        for (int h = 0; h < 2; ++h) {
            CK(mohid::tile_costs(b->cflag.p, b->kfloor.p, L, b->tilesX, b->ntiles[h], mohid::kTileRows[h],
                                 b->tcost[h].p, s));
            CK(cudaMemcpyAsync(b->hcost[h], b->tcost[h].p, sizeof(int) * b->ntiles[h], cudaMemcpyDeviceToHost, s));
        }
        CK(mohid::obc_columns(b->cflag.p, L, b->obcnt.p, b->obcol.p, s));
        // tiles left out of a schedule keep no stale mass-fixer sums
        CK(cudaMemsetAsync(b->mpart.p, 0, sizeof(double) * (size_t)b->nt * b->ntiles[1], s));
    }
    b->packingMasks = masks;
    b->packingMask = in->maskVersion;
    if (masks) b->nfApplied = 0;                 // the flags formed again hold no NoFlux bits
    b->packingRef = b->hasRef;
    CK(cudaMemcpyAsync(&b->hp->moving, b->moving.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&b->hp->vchanged, b->vchanged.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    b->hp->cont = -1.0;
    b->hp->contDT = b->checkedDT;
    if (cdt > 0.0)                                      // continuity for the DT of the last step
        CK(cudaMemcpyAsync(&b->hp->cont, b->scratch.p + 5, sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaEventRecord(b->packEv, s));
    // tensor maps of the shared fields and of the tracer buffers (host only)
    for (int h = 0; h < 2; ++h) {
        const int ty = mohid::kTileRows[h];
        int box[mohid::kNumMaps][4];
        mohid::batched_boxes(hq, hk, 1, ty, box);
        const CUtensorMapDataType tq = hq ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
        const CUtensorMapDataType tk = hk ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
        const int eq = hq ? 2 : 4, ek = hk ? 2 : 4;
        const void* qx = hq ? (const void*)b->Qx16.p : (const void*)b->Qx32.p;
        const void* qy = hq ? (const void*)b->Qy16.p : (const void*)b->Qy32.p;
        const void* qz = hq ? (const void*)b->Qz16.p : (const void*)b->Qz32.p;
        const void* vis = hk ? (const void*)b->Vis16.p : (const void*)b->Vis32.p;
        const void* dif = hk ? (const void*)b->Dif16.p : (const void*)b->Dif32.p;
        bool okm = true;
        mohid::TmaMaps& M = b->maps[h];
        okm &= encode_map(&M.F, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, b->fflag.p, L, 1, box[1]);
        okm &= encode_map(&M.V, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, b->RV.p, L, 1, box[2]);
        okm &= encode_map(&M.Vis, tk, ek, vis, L, 1, box[3]);
        okm &= encode_map(&M.QX, tq, eq, qx, L, 1, box[4]);
        okm &= encode_map(&M.AU, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, b->AreaU.p, L, 1, box[5]);
        okm &= encode_map(&M.QY, tq, eq, qy, L, 1, box[6]);
        okm &= encode_map(&M.AV, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, b->AreaV.p, L, 1, box[7]);
        okm &= encode_map(&M.Vo, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, b->DVR.p, L, 1, box[8]);
        okm &= encode_map(&M.Qz, tq, eq, qz, L, 1, box[9]);
        okm &= encode_map(&M.Dv, tk, ek, dif, L, 1, box[10]);
        okm &= encode_map(&M.Dz, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, b->DZZ.p, L, 1, box[11]);
        okm &= encode_map(&M.Fn, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, b->flag.p, L, 1, box[12]);
        const int gs[5] = {1, 2, 4, 8, 10};
        for (int buf = 0; buf < 2; ++buf)
            for (int g = 0; g < 5; ++g) {
                if (gs[g] > b->nt) continue;
                int bb[mohid::kNumMaps][4];
                mohid::batched_boxes(hq, hk, gs[g], ty, bb);
                okm &= encode_map(&b->mapP[h][buf][g], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
                                  buf ? b->PB.p : b->PA.p, L, b->nt, bb[0], 4);
            }
        if (!okm) return fail(MOHID_AD_ERR_CUDA, stat, "cuTensorMapEncodeTiled failed");
    }
    b->mapsOk = true;
    b->packPending = true;
    b->packingVersion = in->hydroVersion;
    return ok(stat);
}

// Wait for an enqueued repack and take its host-side results: FP16 scales,
// static or moving volumes, the mass fixer's validity, the tile schedule and
// the precomputed continuity check.
int pack_finalize(Batch* b, int* stat)
{
    if (!b->packPending) return ok(stat);
    cudaStream_t s = b->in->stream;
    CK(cudaEventSynchronize(b->packEv));
    b->packPending = false;
    const Batch::PackHost& h = *b->hp;
    if (b->storage >= 1) { b->qsx = h.scale[0]; b->qsy = h.scale[1]; b->qsz = h.scale[2]; }
    if (b->storage >= 2) { b->ksh = h.scale[3]; b->ksv = h.scale[4]; }
    b->staticVol = h.moving == 0;
    // the fixer keeps the masses of tracers loaded under this state; a volume
    // change (or moving volumes) ends it for tracers loaded before
    if (h.moving || (h.vchanged && b->packedOnce))
        for (int t = 0; t < b->nt; ++t)
            if (b->targetVersion[t] != b->packingVersion) {
                const double nan = std::nan("");
                CK(cudaMemcpyAsync(b->mfix.p + 1 + t, &nan, sizeof(double), cudaMemcpyHostToDevice, s));
                CK(cudaMemcpyAsync(b->mfix.p + 1 + 3 * b->nt + t, &nan, sizeof(double), cudaMemcpyHostToDevice, s));
                CK(cudaStreamSynchronize(s));
            }
    b->packedOnce = true;
    b->packedMask = b->packingMask;
    if (!b->packingMasks) {                      // the masks, and with them the schedule, are unchanged
        b->preCont = h.cont;
        b->preContDT = h.contDT;
        b->preContVersion = b->packingVersion;
        b->preContRef = b->packingRef;
        b->packed = true;
        b->packedVersion = b->packingVersion;
        return ok(stat);
    }
    // tile schedules of both heights: tiles holding water, most layers first
    // (stable by tile index)
    for (int h = 0; h < 2; ++h) {
        const int* hc = b->hcost[h];
        std::vector<int> order;
        for (int q = 0; q < b->ntiles[h]; ++q)
            if (hc[q] > 0) order.push_back(q);
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return hc[x] > hc[y]; });
        std::vector<int2> list(order.size());
        for (size_t q = 0; q < order.size(); ++q) list[q] = make_int2(order[q] % b->tilesX, order[q] / b->tilesX);
        b->ntl[h] = (int)list.size();
        if (b->ntl[h])
            CK(cudaMemcpy(b->tl[h].p, list.data(), sizeof(int2) * list.size(), cudaMemcpyHostToDevice));
    }
    b->sumsTh = -1;                              // the memset above cleared the per-tile sums
    b->preCont = h.cont;
    b->preContDT = h.contDT;
    b->preContVersion = b->packingVersion;
    b->preContRef = b->packingRef;
    b->packed = true;
    b->packedVersion = b->packingVersion;
    return ok(stat);
}

// the batched layout holds the instance's current hydrodynamics
int ensure_packed(Batch* b, int* stat)
{
    Instance* in = b->in;
    if (b->packed && b->packedVersion == in->hydroVersion && !b->packPending) return ok(stat);
    if (!b->packPending || b->packingVersion != in->hydroVersion) {
        if (b->packPending) {                    // an older state still in flight
            int c = pack_finalize(b, stat);
            if (c) return c;
        }
        int c = pack_enqueue(b, stat);
        if (c) return c;
    }
    return pack_finalize(b, stat);
}

// the packed flags carry the step's NoAdvFlux / NoDifFlux (after ensure_packed)
int ensure_noflux(Batch* b, const mohid_ad_params* p, int* stat)
{
    Instance* in = b->in;
    const int want = (p->NoAdvFlux ? 1 : 0) | (p->NoDifFlux ? 2 : 0);
    if (want && !in->hasNoFlux)
        return fail(MOHID_AD_ERR_NULLPTR, stat, "NoAdvFlux / NoDifFlux need the NoFluxU/V/W masks (mohid_ad_set_noflux)");
    if (want == b->nfApplied && (want == 0 || b->nfVersion == in->nofluxVersion)) return ok(stat);
    CK(mohid::noflux_flags(in->OP.p, in->CFU.p, in->CFV.p, want ? in->NFU.p : nullptr, want ? in->NFV.p : nullptr,
                           want ? in->NFW.p : nullptr, in->KFloor.p, (want & 1) != 0, (want & 2) != 0, b->flag.p,
                           b->fflag.p, b->L, in->stream));
    b->nfApplied = want;
    b->nfVersion = in->nofluxVersion;
    return ok(stat);
}

// sums: the launch accumulates the mass fixer's per-tile sums (when the fixer runs)
mohid::BatchArgs make_bargs(Batch* b, const mohid_ad_params* p, int t0, int nt, const float* Pin, float* Pout,
                            bool sums = true)
{
    Instance* in = b->in;
    mohid::BatchArgs a;
    std::memset(&a, 0, sizeof a);                // padding too: ensembles compare argument tables bytewise
    a.L = b->L;
    const bool hq = b->storage >= 1, hk = b->storage >= 2;
    a.Qx = hq ? (const void*)b->Qx16.p : (const void*)b->Qx32.p;
    a.Qy = hq ? (const void*)b->Qy16.p : (const void*)b->Qy32.p;
    a.Qz = hq ? (const void*)b->Qz16.p : (const void*)b->Qz32.p;
    a.qsx = b->qsx; a.qsy = b->qsy; a.qsz = b->qsz;
    a.RV = b->RV.p; a.DVR = b->DVR.p;
    a.ViscH = hk ? (const void*)b->Vis16.p : (const void*)b->Vis32.p;
    a.DiffV = hk ? (const void*)b->Dif16.p : (const void*)b->Dif32.p;
    a.ksh = b->ksh; a.ksv = b->ksv;
    a.AreaU = b->AreaU.p; a.AreaV = b->AreaV.p; a.DZZ = b->DZZ.p;
    a.flag = b->flag.p;
    a.fflag = b->fflag.p;
    a.fc = b->fc.p; a.areaCol = b->areaCol.p; a.kfloor = b->kfloor.p; a.cflag = b->cflag.p;
    a.ts = b->L.n3;
    a.Pin = Pin + (long long)t0 * a.ts;
    a.Pout = Pout + (long long)t0 * a.ts;
    a.nt = nt;
    a.t0 = t0;
    a.rk = b->L.nk + 2;
    a.rts = (long long)b->in->nbcols * a.rk;
    a.Ref = b->hasRef ? b->Ref.p + (long long)t0 * a.rts : nullptr;
    a.refIdx = b->hasRef ? b->refIdx.p : nullptr;
    a.W = b->Wsc.p;
    a.G = b->Gsc.p;
    a.Vhi = b->Vhi.p;
    a.Vlo = b->Vlo.p;
    a.mfix = b->mfix.p;
    a.mpart = sums && fix_active(b) ? b->mpart.p : nullptr;
    a.obpart = fix_active(b) && b->hasRef ? b->obpart.p : nullptr;
    a.nob = mohid::kObcBlocks;
    a.tilesX = b->tilesX;
    a.ntiles = b->ntiles[b->ensemble ? 0 : b->th];   // ensembles walk 8-row tiles
    a.ntAll = b->nt;
    a.DT = (float)p->DTProp;
    a.schmidtH = (float)p->schmidt_H;
    a.coefV = (float)p->SchmidtCoef_V;
    a.backV = (float)p->SchmidtBackground_V;
    a.tdec = (float)(1.0 / (1.0 + p->DecayTime / p->DTProp));
    a.nullDif = p->NullDif != 0;
    a.vertical1D = p->Vertical1D != 0;
    a.xzflow = p->XZFlow != 0;
    a.status = in->status.p;
    a.bc = p->BoundaryCondition;
    a.dStart = b->dischOn ? b->dStart.p : nullptr;
    a.dTerms = b->dischOn ? b->dTerms.p : nullptr;
    a.dConc = b->dischOn ? b->dConc.p : nullptr;
    a.DWZ = in->DWZ.p;
    return a;
}

// Decide whether tracers may stay stored as anomalies for this step; convert
// them (and their references) back to absolute values if not.
int ensure_shift_valid(Batch* b, const mohid_ad_params* p, int* stat)
{
    Instance* in = b->in;
    cudaStream_t s = in->stream;
    // without references the boundary columns get ordinary rows, whose budget
    // must close like any other cell's: the check then covers them in full.
    // Discharges are sources the constant does not follow, and faces without
    // advection (NoAdvFlux) break the budget of their cells: absolute values.
    const int flags = (p->XZFlow ? 1 : 0) | (p->Vertical1D ? 2 : 0) | (b->hasRef ? 4 : 0) | (b->dischOn ? 8 : 0) |
                      (p->NoAdvFlux ? 16 : 0);
    if (b->checkedVersion != in->hydroVersion || b->checkedDT != p->DTProp || b->checkedFlags != flags) {
        bool okc = (flags & 27) == 0;
        if (okc && b->preContVersion == in->hydroVersion && b->preContDT == p->DTProp && b->preCont >= 0.0 &&
            b->preContRef == b->hasRef) {
            okc = b->preCont <= 0.0;             // computed with the repack
        } else if (okc) {
            CK(mohid::continuity_residual(in->Qx.p, in->Qy.p, in->Qz.p, in->V.p, in->Vold.p, in->OP.p,
                                          in->CFU.p, in->CFV.p, in->CFW.p, b->hasRef ? in->BP2D.p : nullptr,
                                          p->DTProp, kContinuityTol, b->L, b->scratch.p, s));
            CK(cudaMemcpyAsync(b->hmass, b->scratch.p, sizeof(double), cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            okc = *b->hmass <= 0.0;
        }
        b->shiftOk = okc;
        b->checkedVersion = in->hydroVersion;
        b->checkedDT = p->DTProp;
        b->checkedFlags = flags;
    }
    if (!b->shiftOk) {
        CK(fix_fold(b));                         // constants as corrected by the mass fixer
        bool conv = false;
        for (int t = 0; t < b->nt; ++t) {
            if (b->shift[t] == 0.0) continue;
            conv = true;
            const long long off = (long long)t * b->L.n3;
            CK(mohid::unshift(b->PA.p + off, b->flag.p, b->shift[t], b->L.n3, s));
            CK(mohid::unshift(b->PB.p + off, b->flag.p, b->shift[t], b->L.n3, s));
            if (b->hasRef && t < (int)b->refShift.size() && b->refShift[t] != 0.0) {
                const long long rts = (long long)in->nbcols * (b->L.nk + 2);
                CK(mohid::unshift_ref(b->Ref.p + (long long)t * rts, in->WP.p, in->bcols.p, in->nbcols, in->ni,
                                      in->nj, in->nk, b->refShift[t], s));
                b->refShift[t] = 0.0;
            }
            b->shift[t] = 0.0;
        }
        if (conv) {
            // the fixer's copy of the constants follows (after the fold the
            // corrections are zero): a later fold must not bring the old
            // constants back onto absolute values
            std::vector<double> zero((size_t)b->nt, 0.0);
            CK(cudaMemcpyAsync(b->mfix.p + 1 + b->nt, zero.data(), sizeof(double) * zero.size(),
                               cudaMemcpyHostToDevice, s));
            CK(cudaStreamSynchronize(s));
        }
    }
    return ok(stat);
}

// tracers of the next launch: groups of b->split (10, 8, 4 or 2), then 8, 4, 2, 1
inline int group_size(const Batch* b, int left)
{
    if (left >= 10 && b->split >= 10) return 10;
    if (left >= 8 && b->split >= 8) return 8;
    if (left >= 4 && b->split >= 4) return 4;
    return left >= 2 ? 2 : 1;
}

inline int map_index(int g) { return g == 10 ? 4 : (g == 8 ? 3 : (g == 4 ? 2 : (g == 2 ? 1 : 0))); }

int launches_per_step(const Batch* b)
{
    int n = 0;
    for (int left = b->nt; left > 0; left -= group_size(b, left)) ++n;
    if (fix_active(b) && b->hasRef) n += 2;          // boundary flux, fixer
    else if (b->hasRef) n += 1;                      // targets dropped
    return n;
}

// launches made once per step call: the closed-domain fixer's finish
int launches_per_call(const Batch* b)
{
    return fix_active(b) && !b->hasRef ? 1 : 0;
}

// One transport step of every tracer.  real == false (the autotuner): the step
// writes the other buffer and the scratch only -- no mass-fixer update, no
// parity flip -- so the tracer state is unchanged.
// last: the final step of a step call.  The correction to the tracers'
// constant is held during a call: the stored anomalies evolve independently of
// it on closed domains, and with open boundaries the reference is shifted by
// the same held value.  The correction that brings the mass to its target then
// depends only on the anomalies' sum after the last step, so only that step
// accumulates the sums and corrects.  With open boundaries the target follows
// every step's boundary flux (with the held correction).
cudaError_t enqueue_step(Batch* b, const mohid_ad_params* p, cudaStream_t s, bool real = true, bool last = true)
{
    const bool sums = last;
    const float* Pin = b->cur_in();
    float* Pout = b->cur_out();
    const int h = b->th;
    const int2* tiles = (b->sched == 1 && b->ntl[h] > 0) ? b->tl[h].p : nullptr;
    int t0 = 0;
    while (t0 < b->nt) {
        const int g = group_size(b, b->nt - t0);
        mohid::BatchArgs a = make_bargs(b, p, t0, g, Pin, Pout, sums);
        mohid::TmaMaps m = b->maps[h];
        m.P = b->mapP[h][b->cur ? 1 : 0][map_index(g)];
        cudaError_t e = mohid::launch_batched(a, m, p->AdvMethodH, p->TVDLimitationH, b->storage >= 1,
                                              b->storage >= 2, tiles, b->ntl[h], mohid::kTileRows[h], s);
        if (e != cudaSuccess) return e;
        t0 += g;
    }
    // ImposeNullGradient after the solve, whether or not a reference is given (AD:1874-1880)
    if (p->BoundaryCondition == MOHID_BC_NULL_GRADIENT) {
        Instance* in = b->in;
        cudaError_t e = mohid::null_gradient_batched(Pout, b->L.n3, b->nt, b->flag.p, in->bcols.p, in->nbcols,
                                                     in->KFloor.p, b->L, s);
        if (e != cudaSuccess) return e;
    }
    // Prop_CyclicBoundary after the solve (AD:1874-1880); the walk gave the
    // boundary rows their old values, as for NullGradient
    if (p->BoundaryCondition == MOHID_BC_CYCLIC && b->hasRef) {
        Instance* in = b->in;
        const int rk = b->L.nk + 2;
        cudaError_t e = mohid::cyclic_batched(Pout, b->L.n3, b->nt, b->Ref.p, (long long)in->nbcols * rk, rk,
                                              b->mfix.p + 1 + 2 * b->nt, in->bcols.p, in->nbcols, in->BP2D.p,
                                              in->KFloor.p, b->L, s);
        if (e != cudaSuccess) return e;
    }
    if (!real) return cudaSuccess;
    if (fix_active(b) && (sums || b->hasRef)) {
        cudaError_t e = cudaSuccess;
        if (b->hasRef)                           // the target follows the boundary flux
            e = mohid::obc_flux(make_bargs(b, p, 0, b->nt, Pin, Pout), b->obcol.p, b->storage >= 1, s);
        if (e == cudaSuccess)
            e = mohid::mass_fix_step(sums ? b->mpart.p : nullptr, b->ntiles[h], b->nt, b->mfix.p,
                                     b->hasRef ? b->obpart.p : nullptr, mohid::kObcBlocks, s);
        if (e != cudaSuccess) return e;
    } else if (!fix_active(b) && b->hasRef) {
        // a boundary flux the targets did not follow: they no longer apply
        cudaError_t e = mohid::mass_fix_drop(b->mfix.p, b->nt, s);
        if (e != cudaSuccess) return e;
    }
    b->cur = !b->cur;
    return cudaSuccess;
}

// Autotuner: time every candidate launch schedule (one CTA per tile, or the
// persistent tile list), tile height (8 or 4 rows of 32 columns) and tracer
// grouping (4 or 2 per launch when there are 4 or more tracers, 8 and 10 with
// as many) on the batch itself -- a warm-up step and two timed steps each,
// which leave the tracer state as it was -- in two rounds over all the
// candidates, and keep the one with the fastest of its two times (a single
// round let clock ramp-up or one slow measurement pick a slower schedule).
int autotune(Batch* b, const mohid_ad_params* p, int* stat)
{
    cudaStream_t s = b->in->stream;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    struct Cand { int split, h, sched; float ms; };
    std::vector<Cand> cands;
    for (int split : {10, 8, 4, 2}) {
        if ((split == 10 && b->nt < 10) || (split == 8 && b->nt < 8) || (split == 2 && b->nt < 4)) continue;
        for (int h = 0; h < 2; ++h)
            for (int sched : {0, 1})
                if (sched == 0 || b->ntl[h] > 0) cands.push_back({split, h, sched, 1e30f});
    }
    cudaError_t err = cudaSuccess;
    for (int round = 0; round < 2 && err == cudaSuccess; ++round)
        for (Cand& c : cands) {
            b->sched = c.sched;
            b->split = c.split;
            b->th = c.h;
            err = enqueue_step(b, p, s, false, false);
            if (err == cudaSuccess) err = cudaEventRecord(e0, s);
            for (int r = 0; r < 2 && err == cudaSuccess; ++r) err = enqueue_step(b, p, s, false, false);
            if (err == cudaSuccess) err = cudaEventRecord(e1, s);
            if (err == cudaSuccess) err = cudaEventSynchronize(e1);
            float ms = 0.f;
            if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
            if (err != cudaSuccess) break;
            c.ms = std::min(c.ms, ms);
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    Cand best{4, 0, 0, 1e30f};
    for (const Cand& c : cands)
        if (c.ms < best.ms) best = c;
    b->sched = best.sched;
    b->split = best.split;
    b->th = best.h;
    if (err != cudaSuccess) return fail(MOHID_AD_ERR_CUDA, stat, cuda_msg("autotune", err));
    b->tuned = true;
    return ok(stat);
}

// ---- ensembles --------------------------------------------------------------
struct Ensemble {
    std::vector<Batch*> m;
    std::vector<int> bids;
    int nt = 0;
    int device = 0;
    cudaStream_t s = nullptr;
    DevBuf<mohid::BatchArgs> dA;         // [2][2][n]: arguments per buffer parity, without / with the
                                         // closed-domain fixer's sums (a call's last step)
    DevBuf<mohid::TmaMaps> dM;           // [2][n]
    DevBuf<int4> tiles;                  // (member, bx, by, 0), costliest first
    int ntiles = 0;
    std::vector<mohid::BatchArgs> hA;    // what dA holds
    std::vector<mohid::TmaMaps> hM;
    bool uploaded = false;
    bool cur = false;                    // buffer parity of every member
    cudaGraphExec_t graph = nullptr;
    int graphSteps = 0;
    bool graphCur = false;
    int graphMethod = 0, graphLimiter = 0;
    bool graphLast = false;
    void release()
    {
        dA.release(); dM.release(); tiles.release();
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
    }
};

std::map<int, Ensemble*> g_ens;
int g_next_eid = 1;

Ensemble* elookup(const int* eid)
{
    if (!eid) return nullptr;
    std::lock_guard<std::mutex> lk(g_bmu);
    auto it = g_ens.find(*eid);
    return it == g_ens.end() ? nullptr : it->second;
}

// One step of every member: one launch over all tiles, then every parity
// flips.  last: the final step of the call, after which the members' mass
// fixer corrects (members with open boundaries follow their boundary flux
// every step).
cudaError_t enqueue_ens_step(Ensemble* E, int method, int limiter, int grid, bool last)
{
    const size_t n = E->m.size();
    const size_t moff = E->cur ? n : 0;
    const size_t aoff = ((E->cur ? 2 : 0) + (last ? 1 : 0)) * n;
    const bool open = std::any_of(E->m.begin(), E->m.end(), [](const Batch* b) { return b->hasRef; });
    cudaError_t e = mohid::launch_ensemble(E->dA.p + aoff, E->dM.p + moff, E->tiles.p, E->ntiles, grid, E->nt,
                                           method, limiter, open, E->s);
    bool fix = false;
    for (size_t q = 0; q < n && e == cudaSuccess; ++q) {
        Batch* b = E->m[q];
        fix |= fix_active(b) && (last || b->hasRef);   // records without sums or flux return
        if (!b->hasRef) continue;
        if (fix_active(b)) e = mohid::obc_flux(E->hA[aoff + q], b->obcol.p, false, E->s);
        else e = mohid::mass_fix_drop(b->mfix.p, b->nt, E->s);
    }
    if (e == cudaSuccess && fix) e = mohid::mass_fix_step_many(E->dA.p + aoff, (int)n, E->nt, E->s);
    E->cur = !E->cur;
    return e;
}

}  // namespace
}  // namespace mohid_abi

using namespace mohid_abi;

extern "C" {

int mohid_ad_batched_create(int* bid, const int* id, const int* ntracers, const int* storage, int* stat)
{
    TraceRange trace_("mohid_ad_batched_create");
    if (!bid || !ntracers || !storage) return fail(MOHID_AD_ERR_NULLPTR, stat, "mohid_ad_batched_create: NULL argument");
    Instance* in = lookup(id);
    if (!in) return fail(MOHID_AD_ERR_ID, stat, "unknown plain instance id");
    if (*ntracers < 1) return fail(MOHID_AD_ERR_BOUNDS, stat, "ntracers must be >= 1");
    if (*storage < 0 || *storage > 2) return fail(MOHID_AD_ERR_OPTION, stat, "storage must be 0, 1 or 2");
    if (in->nk > 200) return fail(MOHID_AD_ERR_UNSUPPORTED, stat, "KUB > 200 layers not supported");
    CK(cudaSetDevice(in->device));
    Batch* b = new Batch();
    b->plain = *id;
    b->in = in;
    b->nt = *ntracers;
    b->storage = *storage;
    b->L = mohid::make_layout(in->ni, in->nj, in->nk);
    const size_t n3 = (size_t)b->L.n3, n2 = (size_t)b->L.n2;
    auto bad = [&](cudaError_t e, const char* what) {
        std::string m = cuda_msg(what, e);
        b->release();
        delete b;
        return fail(e == cudaErrorMemoryAllocation ? MOHID_AD_ERR_ALLOC : MOHID_AD_ERR_CUDA, stat, m);
    };
    cudaError_t e;
    if (b->storage >= 1) {
        DevBuf<__half>* h[] = {&b->Qx16, &b->Qy16, &b->Qz16};
        for (auto* x : h) if ((e = x->alloc(n3)) != cudaSuccess) return bad(e, "cudaMalloc");
    } else {
        DevBuf<float>* f[] = {&b->Qx32, &b->Qy32, &b->Qz32};
        for (auto* x : f) if ((e = x->alloc(n3)) != cudaSuccess) return bad(e, "cudaMalloc");
    }
    if (b->storage >= 2) {
        DevBuf<__half>* h[] = {&b->Vis16, &b->Dif16};
        for (auto* x : h) if ((e = x->alloc(n3)) != cudaSuccess) return bad(e, "cudaMalloc");
    } else {
        DevBuf<float>* f[] = {&b->Vis32, &b->Dif32};
        for (auto* x : f) if ((e = x->alloc(n3)) != cudaSuccess) return bad(e, "cudaMalloc");
    }
    DevBuf<float>* f3[] = {&b->AreaU, &b->AreaV, &b->DZZ};
    for (auto* x : f3) if ((e = x->alloc(n3)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = b->RV.alloc(n3)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = b->DVR.alloc(n3)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = b->flag.alloc(n3)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = b->fflag.alloc(n3)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = b->cflag.alloc(n2)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = b->fc.alloc(2 * n2)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = b->areaCol.alloc(n2)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = b->kfloor.alloc(n2)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = b->PA.alloc(n3 * b->nt)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = b->PB.alloc(n3 * b->nt)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = b->Wsc.alloc(n3)) != cudaSuccess) return bad(e, "cudaMalloc");
    {
        // the largest tracer group a launch can hold (group_size): NT floats of G per cell
        const int gmax = b->nt >= 10 ? 10 : (b->nt >= 8 ? 8 : (b->nt >= 4 ? 4 : (b->nt >= 2 ? 2 : 1)));
        if ((e = b->Gsc.alloc(n3 * (size_t)gmax)) != cudaSuccess) return bad(e, "cudaMalloc");
    }
    b->tilesX = (in->ni + mohid::kTX - 1) / mohid::kTX;
    for (int h = 0; h < 2; ++h)
        b->ntiles[h] = b->tilesX * ((in->nj + mohid::kTileRows[h] - 1) / mohid::kTileRows[h]);
    if ((e = b->Vhi.alloc(n3)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = b->Vlo.alloc(n3)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = b->mfix.alloc(1 + 4 * (size_t)b->nt)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = b->obpart.alloc((size_t)(b->nt + 1) * mohid::kObcBlocks)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = b->obcol.alloc(n2 + 1)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = b->obcnt.alloc(mohid::kObcBlocks)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = b->mpart.alloc((size_t)b->nt * b->ntiles[1])) != cudaSuccess) return bad(e, "cudaMalloc");
    for (int h = 0; h < 2; ++h) {
        if ((e = cudaMallocHost((void**)&b->hcost[h], sizeof(int) * (size_t)b->ntiles[h])) != cudaSuccess)
            return bad(e, "cudaMallocHost");
        if ((e = b->tl[h].alloc(b->ntiles[h])) != cudaSuccess) return bad(e, "cudaMalloc");
        if ((e = b->tcost[h].alloc(b->ntiles[h])) != cudaSuccess) return bad(e, "cudaMalloc");
    }
    if ((e = b->moving.alloc(1)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = b->Vprev.alloc(in->n3)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = b->partial.alloc(2 * kMassBlocks)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = b->vpart.alloc(2 * kPackBlocks)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = b->scratch.alloc(8)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = b->tscratch.alloc(4)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = b->tpartial.alloc(2 * kMassBlocks)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = b->dscale.alloc(5)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = b->dinv.alloc(5)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = b->vchanged.alloc(1)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = cudaStreamCreateWithFlags(&b->cs, cudaStreamNonBlocking)) != cudaSuccess) return bad(e, "cudaStreamCreate");
    if ((e = cudaEventCreateWithFlags(&b->packEv, cudaEventDisableTiming)) != cudaSuccess)
        return bad(e, "cudaEventCreate");
    if ((e = cudaMallocHost((void**)&b->hp, sizeof(Batch::PackHost))) != cudaSuccess) return bad(e, "cudaMallocHost");
    b->targetVersion.assign(b->nt, ~0u);
    if ((e = b->stage.alloc(in->n3)) != cudaSuccess) return bad(e, "cudaMalloc");
    b->shift.assign(b->nt, 0.0);
    if ((e = cudaMallocHost((void**)&b->hmass, 4 * sizeof(double))) != cudaSuccess) return bad(e, "cudaMallocHost");
    {
        std::lock_guard<std::mutex> lk(g_bmu);
        *bid = g_next_bid++;
        g_batch[*bid] = b;
    }
    return ok(stat);
}

int mohid_ad_batched_pack_hydro(const int* bid, int* stat)
{
    TraceRange trace_("mohid_ad_batched_pack_hydro");
    Batch* b = blookup(bid);
    if (!b) return fail(MOHID_AD_ERR_ID, stat, "unknown batch id");
    CK(cudaSetDevice(b->in->device));
    b->fluxLast = false;                         // the fluxes read the packed fields of their step
    return ensure_packed(b, stat);
}

int mohid_ad_batched_set_tracer(const int* bid, const int* t, const double* PROP, const int* on_device, int* stat)
{
    TraceRange trace_("mohid_ad_batched_set_tracer");
    Batch* b = blookup(bid);
    if (!b) return fail(MOHID_AD_ERR_ID, stat, "unknown batch id");
    if (!t || !PROP || !on_device) return fail(MOHID_AD_ERR_NULLPTR, stat, "NULL argument");
    if (*t < 0 || *t >= b->nt) return fail(MOHID_AD_ERR_BOUNDS, stat, "tracer index out of range");
    b->fluxLast = false;                         // the buffers no longer hold the last step's fields
    Instance* in = b->in;
    if (!in->hydro) return fail(MOHID_AD_ERR_OPTION, stat, "the plain instance has no hydrodynamics set");
    CK(cudaSetDevice(in->device));
    cudaStream_t s = in->stream;
    // earlier work on the tracer buffers (a step) comes first; a new
    // hydrodynamic state starts repacking on the instance's stream meanwhile
    cudaEvent_t before;
    CK(cudaEventCreateWithFlags(&before, cudaEventDisableTiming));
    cudaError_t ev = cudaEventRecord(before, s);
    if (ev == cudaSuccess) ev = cudaStreamWaitEvent(b->cs, before, 0);
    cudaEventDestroy(before);
    if (ev != cudaSuccess) return fail(MOHID_AD_ERR_CUDA, stat, cuda_msg("cudaStreamWaitEvent", ev));
    if ((!b->packed || b->packedVersion != in->hydroVersion) &&
        !(b->packPending && b->packingVersion == in->hydroVersion)) {
        if (b->packPending) {
            int c = pack_finalize(b, stat);
            if (c) return c;
        }
        int c = pack_enqueue(b, stat);
        if (c) return c;
    }
    cudaStream_t ts = b->cs;
    const double* src = PROP;
    if (!*on_device) {
        CK(cudaMemcpyAsync(b->stage.p, PROP, sizeof(double) * in->n3, cudaMemcpyHostToDevice, ts));
        src = b->stage.p;
    }
    const long long off = (long long)*t * b->L.n3;
    // shift = mean over the water cells, rounded to an FP32 value
    CK(mohid::water_mean(src, in->WP.p, b->L, b->tpartial.p, kMassBlocks, b->tscratch.p, ts));
    CK(cudaMemcpyAsync(b->hmass + 1, b->tscratch.p, sizeof(double), cudaMemcpyDeviceToHost, ts));
    CK(cudaStreamSynchronize(ts));
    double sh = std::isfinite(b->hmass[1]) ? (double)(float)b->hmass[1] : 0.0;
    b->shift[*t] = sh;
    CK(mohid::pack_tracer(src, b->PA.p + off, b->PB.p + off, in->KFloor.p, in->WP.p, sh, b->L, ts));
    // the mass fixer keeps the FP64 mass of the field as loaded (with the volume it starts the step in)
    CK(mohid::mass_fix_load(src, in->Vold.p, in->WP.p, b->L, b->tpartial.p, kMassBlocks, sh, *t, b->nt,
                            b->mfix.p, ts));
    b->fixDirty = true;
    b->targetVersion[*t] = in->hydroVersion;
    CK(cudaStreamSynchronize(ts));
    return ok(stat);
}

int mohid_ad_batched_get_tracer(const int* bid, const int* t, double* PROP, const int* on_device, int* stat)
{
    TraceRange trace_("mohid_ad_batched_get_tracer");
    Batch* b = blookup(bid);
    if (!b) return fail(MOHID_AD_ERR_ID, stat, "unknown batch id");
    if (!t || !PROP || !on_device) return fail(MOHID_AD_ERR_NULLPTR, stat, "NULL argument");
    if (*t < 0 || *t >= b->nt) return fail(MOHID_AD_ERR_BOUNDS, stat, "tracer index out of range");
    Instance* in = b->in;
    CK(cudaSetDevice(in->device));
    cudaStream_t s = in->stream;
    const long long off = (long long)*t * b->L.n3;
    double* dst = *on_device ? PROP : b->stage.p;
    CK(mohid::unpack_tracer(b->cur_in() + off, dst, nullptr, in->WP.p, in->KFloor.p, b->shift[*t],
                            b->mfix.p + 1 + 2 * b->nt + *t, b->L, s));
    if (!*on_device) {
        CK(cudaMemcpyAsync(PROP, b->stage.p, sizeof(double) * in->n3, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    }
    return ok(stat);
}

// DischConc of tracer t: one value per discharge cell of the plain instance's
// mohid_ad_set_discharges call, in its order (SetDischarges AD:978-1075, called
// per property with the property's concentrations, WP:14763-14770)
int mohid_ad_batched_set_discharge_conc(const int* bid, const int* t, const double* DischConc, int* stat)
{
    TraceRange trace_("mohid_ad_batched_set_discharge_conc");
    Batch* b = blookup(bid);
    if (!b) return fail(MOHID_AD_ERR_ID, stat, "unknown batch id");
    if (!t) return fail(MOHID_AD_ERR_NULLPTR, stat, "NULL argument");
    if (*t < 0 || *t >= b->nt) return fail(MOHID_AD_ERR_BOUNDS, stat, "tracer index out of range");
    Instance* in = b->in;
    if (!in->hasDisch) return fail(MOHID_AD_ERR_OPTION, stat, "the plain instance has no discharges set");
    if (in->nDischCells > 0 && !DischConc) return fail(MOHID_AD_ERR_NULLPTR, stat, "DischConc is NULL");
    if ((int)b->hConc.size() < b->nt) b->hConc.resize(b->nt);
    b->hConc[*t].assign(DischConc, DischConc + in->nDischCells);
    b->dischDirty = true;
    return ok(stat);
}

int mohid_ad_batched_set_reference(const int* bid, const int* t, const double* ReferenceProp,
                                   const int* on_device, int* stat)
{
    TraceRange trace_("mohid_ad_batched_set_reference");
    Batch* b = blookup(bid);
    if (!b) return fail(MOHID_AD_ERR_ID, stat, "unknown batch id");
    if (!t || !ReferenceProp || !on_device) return fail(MOHID_AD_ERR_NULLPTR, stat, "NULL argument");
    if (*t < 0 || *t >= b->nt) return fail(MOHID_AD_ERR_BOUNDS, stat, "tracer index out of range");
    Instance* in = b->in;
    CK(cudaSetDevice(in->device));
    cudaStream_t s = in->stream;
    // only the boundary columns read a reference: one row of nk + 2 layers
    // per boundary column (the reference's sweep order) and tracer
    const long long rts = (long long)in->nbcols * (b->L.nk + 2);
    if (!b->Ref.p) {
        cudaError_t e = b->Ref.alloc((size_t)std::max<long long>(1, rts * b->nt));
        if (e == cudaSuccess) e = b->refIdx.alloc((size_t)b->L.n2);
        if (e != cudaSuccess) {
            b->Ref.release(); b->refIdx.release();
            return fail(MOHID_AD_ERR_ALLOC, stat, cuda_msg("cudaMalloc", e));
        }
        CK(mohid::ref_index(in->bcols.p, in->nbcols, in->ni, b->L, b->refIdx.p, s));
    }
    const double* src = ReferenceProp;
    if (!*on_device) {
        CK(cudaMemcpyAsync(b->stage.p, ReferenceProp, sizeof(double) * in->n3, cudaMemcpyHostToDevice, s));
        src = b->stage.p;
    }
    // stored relative to the tracer's loaded constant, like the tracer; the
    // step subtracts the mass fixer's correction to that constant
    CK(mohid::pack_ref(src, in->WP.p, in->bcols.p, in->nbcols, in->ni, in->nj, in->nk, b->shift[*t],
                       b->Ref.p + (long long)*t * rts, s));
    CK(cudaStreamSynchronize(s));
    b->hasRef = true;
    b->refShift.resize(b->nt, 0.0);
    b->refShift[*t] = b->shift[*t];
    return ok(stat);
}

int mohid_ad_batched_step(const int* bid, const mohid_ad_params* p, const int* nsteps, const int* use_graph,
                          int* stat)
{
    TraceRange trace_("mohid_ad_batched_step");
    Batch* b = blookup(bid);
    if (!b) return fail(MOHID_AD_ERR_ID, stat, "unknown batch id");
    if (!nsteps || !use_graph) return fail(MOHID_AD_ERR_NULLPTR, stat, "NULL argument");
    if (b->ensemble) return fail(MOHID_AD_ERR_OPTION, stat, "the batch is stepped by an ensemble");
    std::string why;
    int code = check_batched_params(p, b->hasRef, why);
    if (code) return fail(code, stat, why);
    if (*nsteps < 1) return fail(MOHID_AD_ERR_BOUNDS, stat, "nsteps must be >= 1");
    CK(cudaSetDevice(b->in->device));
    b->fluxLast = false;                         // set again once the steps are enqueued
    if ((code = ensure_discharges(b, stat)) != 0) return code;
    b->bcFix = bc_fixable(b, p);
    if (b->hasRef)
        for (int t = 0; t < b->nt; ++t)
            if (t >= (int)b->refShift.size() || b->refShift[t] != b->shift[t])
                return fail(MOHID_AD_ERR_OPTION, stat,
                            "set the reference of every tracer after (re)loading the tracer");
    Instance* in = b->in;
    {
        int c = ensure_packed(b, stat);
        if (c) return c;
    }
    CK(cudaSetDevice(in->device));
    {
        int c = ensure_noflux(b, p, stat);
        if (c) return c;
    }
    {
        int c = ensure_shift_valid(b, p, stat);
        if (c) return c;
    }
    cudaStream_t s = in->stream;
    if (!b->tuned) {
        int c = autotune(b, p, stat);
        if (c) return c;
    }
    if (fix_active(b)) b->fixDirty = true;
    // the fixer's per-tile sums are laid out by the tile height in use; the
    // tiles a list schedule leaves out must read zero in that layout
    if (b->sumsTh != -1 && b->sumsTh != b->th)
        CK(cudaMemsetAsync(b->mpart.p, 0, sizeof(double) * (size_t)b->nt * b->ntiles[1], s));
    b->sumsTh = b->th;
    auto done = [&]() {
        b->fluxLast = p->CellFluxes != 0;
        if (b->fluxLast) b->fluxParams = *p;
        return ok(stat);
    };
    if (!*use_graph) {
        for (int n = 0; n < *nsteps; ++n) CK(enqueue_step(b, p, s, true, n == *nsteps - 1));
        return done();
    }
    // CUDA graph of an even number of steps: the ping-pong returns to the
    // buffer it started from, so the graph stays valid for that parity; an
    // odd remainder step is launched directly.
    const int pairs = *nsteps / 2;
    if (pairs > 0) {
        const bool glast = *nsteps % 2 == 0;          // the graph holds the call's last step
        const bool reuse = b->graph && b->graphSteps == 2 * pairs && b->graphCur == b->cur &&
                           b->graphSched == b->sched && b->graphSplit == b->split && b->graphTh == b->th &&
                           b->graphFix == fix_key(b) && b->graphLast == glast &&
                           b->graphPack == b->packedVersion &&
                           b->graphDisch == (b->dischOn ? b->dischUploads : ~0u) &&
                           std::memcmp(&b->graphParams, p, sizeof(*p)) == 0;
        if (!reuse) {
            if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
            const bool cur0 = b->cur;
            cudaGraph_t g;
            CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            cudaError_t e = cudaSuccess;
            for (int n = 0; n < 2 * pairs && e == cudaSuccess; ++n)
                e = enqueue_step(b, p, s, true, glast && n == 2 * pairs - 1);
            cudaError_t e2 = cudaStreamEndCapture(s, &g);
            b->cur = cur0;
            if (e != cudaSuccess) return fail(MOHID_AD_ERR_CUDA, stat, cuda_msg("capture", e));
            if (e2 != cudaSuccess) return fail(MOHID_AD_ERR_CUDA, stat, cuda_msg("cudaStreamEndCapture", e2));
            e = cudaGraphInstantiate(&b->graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) { b->graph = nullptr; return fail(MOHID_AD_ERR_CUDA, stat, cuda_msg("cudaGraphInstantiate", e)); }
            b->graphSteps = 2 * pairs;
            b->graphCur = cur0;
            b->graphParams = *p;
            b->graphSched = b->sched;
            b->graphSplit = b->split;
            b->graphTh = b->th;
            b->graphFix = fix_key(b);
            b->graphLast = glast;
            b->graphPack = b->packedVersion;
            b->graphDisch = b->dischOn ? b->dischUploads : ~0u;
        }
        CK(cudaGraphLaunch(b->graph, s));
    }
    if (*nsteps % 2) CK(enqueue_step(b, p, s, true, true));
    return done();
}

int mohid_ad_batched_autotune(const int* bid, const mohid_ad_params* p, int* stat)
{
    TraceRange trace_("mohid_ad_batched_autotune");
    Batch* b = blookup(bid);
    if (!b) return fail(MOHID_AD_ERR_ID, stat, "unknown batch id");
    if (!p) return fail(MOHID_AD_ERR_NULLPTR, stat, "NULL argument");
    if (b->ensemble) return fail(MOHID_AD_ERR_OPTION, stat, "the batch is stepped by an ensemble");
    std::string why;
    int code = check_batched_params(p, b->hasRef, why);
    if (code) return fail(code, stat, why);
    Instance* in = b->in;
    CK(cudaSetDevice(in->device));
    b->fluxLast = false;
    if ((code = ensure_discharges(b, stat)) != 0) return code;
    {
        int c = ensure_packed(b, stat);
        if (c) return c;
    }
    int c = ensure_noflux(b, p, stat);
    if (c) return c;
    c = ensure_shift_valid(b, p, stat);
    if (c) return c;
    return autotune(b, p, stat);
}

int mohid_ad_batched_set_schedule(const int* bid, const int* sched, const int* split, const int* tile_rows,
                                  int* stat)
{
    Batch* b = blookup(bid);
    if (!b) return fail(MOHID_AD_ERR_ID, stat, "unknown batch id");
    if (!sched || !split) return fail(MOHID_AD_ERR_NULLPTR, stat, "NULL argument");
    if ((*sched != 0 && *sched != 1) || (*split != 10 && *split != 8 && *split != 4 && *split != 2))
        return fail(MOHID_AD_ERR_OPTION, stat, "schedule must be 0 or 1 and split 10, 8, 4 or 2");
    int th = b->th;
    if (tile_rows) {
        if (*tile_rows == mohid::kTileRows[0]) th = 0;
        else if (*tile_rows == mohid::kTileRows[1]) th = 1;
        else return fail(MOHID_AD_ERR_OPTION, stat, "tile_rows must be 8 or 4");
    }
    b->sched = *sched;
    b->split = *split;
    b->th = th;
    b->tuned = true;
    return ok(stat);
}

int mohid_ad_batched_schedule(const int* bid, int* launches, int* sched, int* split, int* per_call,
                              int* tile_rows, int* stat)
{
    Batch* b = blookup(bid);
    if (!b) return fail(MOHID_AD_ERR_ID, stat, "unknown batch id");
    if (launches) *launches = launches_per_step(b);
    if (per_call) *per_call = launches_per_call(b);
    if (sched) *sched = b->sched;
    if (split) *split = b->split;
    if (tile_rows) *tile_rows = mohid::kTileRows[b->th];
    return ok(stat);
}

int mohid_ad_batched_set_mass_fix(const int* bid, const int* on, int* stat)
{
    Batch* b = blookup(bid);
    if (!b) return fail(MOHID_AD_ERR_ID, stat, "unknown batch id");
    if (!on) return fail(MOHID_AD_ERR_NULLPTR, stat, "NULL argument");
    b->massFix = *on != 0;
    return ok(stat);
}

int mohid_ad_batched_mass(const int* bid, const int* t, double* mass, int* stat)
{
    TraceRange trace_("mohid_ad_batched_mass");
    Batch* b = blookup(bid);
    if (!b) return fail(MOHID_AD_ERR_ID, stat, "unknown batch id");
    if (!t || !mass) return fail(MOHID_AD_ERR_NULLPTR, stat, "NULL argument");
    if (*t < 0 || *t >= b->nt) return fail(MOHID_AD_ERR_BOUNDS, stat, "tracer index out of range");
    Instance* in = b->in;
    CK(cudaSetDevice(in->device));
    {
        int c = ensure_packed(b, stat);
        if (c) return c;
    }
    cudaStream_t s = in->stream;
    const float* P = b->cur_in() + (long long)*t * b->L.n3;
    CK(mohid::mass_batched(P, in->V.p, b->flag.p, b->shift[*t], b->mfix.p + 1 + 2 * b->nt + *t, b->L,
                           b->partial.p, kMassBlocks, s));
    CK(mohid::mass_finish(b->partial.p, kMassBlocks, b->scratch.p, s));
    CK(cudaMemcpyAsync(b->hmass, b->scratch.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    *mass = *b->hmass;
    return ok(stat);
}

int mohid_ad_debug_wait_probe(const int* polls, int* stat)
{
    if (!polls) return fail(MOHID_AD_ERR_NULLPTR, stat, "NULL argument");
    if (*polls < 1) return fail(MOHID_AD_ERR_BOUNDS, stat, "polls must be >= 1");
    unsigned* d = nullptr;
    unsigned h = 0;
    cudaError_t e = cudaMalloc((void**)&d, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(d, 0, sizeof(unsigned));
    if (e == cudaSuccess) e = mohid::wait_probe((unsigned)*polls, d, 0);
    if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(unsigned), cudaMemcpyDeviceToHost);
    if (d) cudaFree(d);
    if (e != cudaSuccess) return fail(MOHID_AD_ERR_CUDA, stat, cuda_msg("wait probe", e));
    std::string why;
    const int code = status_to_code(h, why);
    return code ? fail(code, stat, why) : ok(stat);
}

int mohid_ad_batched_boundary_flux(const int* bid, const int* t, double* flux, int* stat)
{
    Batch* b = blookup(bid);
    if (!b) return fail(MOHID_AD_ERR_ID, stat, "unknown batch id");
    if (!t || !flux) return fail(MOHID_AD_ERR_NULLPTR, stat, "NULL argument");
    if (*t < 0 || *t >= b->nt) return fail(MOHID_AD_ERR_BOUNDS, stat, "tracer index out of range");
    Instance* in = b->in;
    CK(cudaSetDevice(in->device));
    cudaStream_t s = in->stream;
    CK(cudaMemcpyAsync(b->hmass, b->mfix.p + 1 + 3 * b->nt + *t, sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    *flux = *b->hmass;
    return ok(stat);
}

// CellFluxes of tracer *t's last step (GetAdvFlux / GetDifFlux, AD:697-860),
// formed from the ping-pong buffers (batched_flux.cu)
static int batched_get_fluxes(const int* bid, const int* t, bool adv, double* X, double* Y, double* Z,
                              const int* on_device, int* stat)
{
    Batch* b = blookup(bid);
    if (!b) return fail(MOHID_AD_ERR_ID, stat, "unknown batch id");
    if (!t || !on_device) return fail(MOHID_AD_ERR_NULLPTR, stat, "NULL argument");
    if (*t < 0 || *t >= b->nt) return fail(MOHID_AD_ERR_BOUNDS, stat, "tracer index out of range");
    if (!b->fluxLast) return fail(MOHID_AD_ERR_OPTION, stat, "the last step was not made with CellFluxes");
    Instance* in = b->in;
    CK(cudaSetDevice(in->device));
    if (!b->fluxOut.p) {
        cudaError_t e = b->fluxOut.alloc((size_t)3 * in->n3);
        if (e != cudaSuccess) return fail(MOHID_AD_ERR_ALLOC, stat, cuda_msg("cudaMalloc", e));
    }
    cudaStream_t s = in->stream;
    const mohid_ad_params& p = b->fluxParams;
    const long long off = (long long)*t * b->L.n3;
    mohid::BatchArgs a = make_bargs(b, &p, 0, b->nt, b->cur_in(), b->cur_out(), false);
    CK(mohid::cell_fluxes_batched(a, b->cur_out() + off, b->cur_in() + off, b->shift[*t],
                                  b->mfix.p + 1 + 2 * b->nt + *t, adv, b->fluxOut.p, (long long)in->n3,
                                  p.AdvMethodH, p.TVDLimitationH, b->storage >= 1, b->storage >= 2, s));
    const cudaMemcpyKind kind = *on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    double* dst[3] = {X, Y, Z};
    for (int q = 0; q < 3; ++q)
        if (dst[q])
            CK(cudaMemcpyAsync(dst[q], b->fluxOut.p + (size_t)q * in->n3, sizeof(double) * in->n3, kind, s));
    CK(cudaStreamSynchronize(s));
    return ok(stat);
}

int mohid_ad_batched_get_adv_flux(const int* bid, const int* t, double* AdvFluxX, double* AdvFluxY,
                                  double* AdvFluxZ, const int* on_device, int* stat)
{
    TraceRange trace_("mohid_ad_batched_get_adv_flux");
    return batched_get_fluxes(bid, t, true, AdvFluxX, AdvFluxY, AdvFluxZ, on_device, stat);
}

int mohid_ad_batched_get_dif_flux(const int* bid, const int* t, double* DifFluxX, double* DifFluxY,
                                  double* DifFluxZ, const int* on_device, int* stat)
{
    TraceRange trace_("mohid_ad_batched_get_dif_flux");
    return batched_get_fluxes(bid, t, false, DifFluxX, DifFluxY, DifFluxZ, on_device, stat);
}

int mohid_ad_batched_sync(const int* bid, int* stat)
{
    Batch* b = blookup(bid);
    if (!b) return fail(MOHID_AD_ERR_ID, stat, "unknown batch id");
    return mohid_ad_sync(&b->plain, stat);
}

int mohid_ad_batched_destroy(int* bid, int* stat)
{
    Batch* b = nullptr;
    if (bid) {
        std::lock_guard<std::mutex> lk(g_bmu);
        auto it = g_batch.find(*bid);
        if (it != g_batch.end()) {
            if (it->second->ensemble) return fail(MOHID_AD_ERR_OPTION, stat, "the batch belongs to an ensemble");
            b = it->second;
            g_batch.erase(it);
        }
    }
    if (!b) return fail(MOHID_AD_ERR_ID, stat, "unknown batch id");
    cudaSetDevice(b->in->device);
    cudaStreamSynchronize(b->in->stream);
    b->release();
    delete b;
    *bid = 0;
    return ok(stat);
}

int mohid_ad_ensemble_create(int* eid, const int* nmembers, const int* bids, int* stat)
{
    if (!eid || !nmembers || !bids) return fail(MOHID_AD_ERR_NULLPTR, stat, "mohid_ad_ensemble_create: NULL argument");
    if (*nmembers < 1) return fail(MOHID_AD_ERR_BOUNDS, stat, "nmembers must be >= 1");
    std::vector<Batch*> m;
    for (int q = 0; q < *nmembers; ++q) {
        Batch* b = blookup(&bids[q]);
        if (!b) return fail(MOHID_AD_ERR_ID, stat, "unknown batch id " + std::to_string(bids[q]));
        if (b->ensemble) return fail(MOHID_AD_ERR_OPTION, stat, "batch " + std::to_string(bids[q]) + " is already in an ensemble");
        if (std::find(m.begin(), m.end(), b) != m.end()) return fail(MOHID_AD_ERR_OPTION, stat, "a batch is listed twice");
        if (b->storage != 0) return fail(MOHID_AD_ERR_UNSUPPORTED, stat, "ensemble members must use FP32 storage");
        if (b->nt != 1 && b->nt != 2 && b->nt != 4)
            return fail(MOHID_AD_ERR_UNSUPPORTED, stat, "ensemble members must hold 1, 2 or 4 tracers");
        if (!m.empty() && b->nt != m[0]->nt) return fail(MOHID_AD_ERR_OPTION, stat, "members hold different tracer counts");
        if (!m.empty() && b->in->device != m[0]->in->device) return fail(MOHID_AD_ERR_OPTION, stat, "members on different devices");
        if (!m.empty() && b->cur != m[0]->cur) return fail(MOHID_AD_ERR_OPTION, stat, "members at different buffer parities");
        m.push_back(b);
    }
    CK(cudaSetDevice(m[0]->in->device));
    Ensemble* E = new Ensemble();
    E->m = m;
    E->bids.assign(bids, bids + *nmembers);
    E->nt = m[0]->nt;
    E->device = m[0]->in->device;
    E->s = m[0]->in->stream;
    E->cur = m[0]->cur;
    // tiles of every member, the deepest domains first (a tile's cost grows with its layers)
    std::vector<int4> t;
    for (int q = 0; q < (int)m.size(); ++q) {
        const mohid::BLayout& L = m[q]->L;
        const int gx = (L.ni + mohid::kTX - 1) / mohid::kTX, gy = (L.nj + mohid::kTY - 1) / mohid::kTY;
        for (int by = 0; by < gy; ++by)
            for (int bx = 0; bx < gx; ++bx) t.push_back(make_int4(q, bx, by, 0));
    }
    std::stable_sort(t.begin(), t.end(), [&](const int4& a, const int4& b) { return m[a.x]->L.nk > m[b.x]->L.nk; });
    E->ntiles = (int)t.size();
    const size_t n = m.size();
    cudaError_t e;
    if ((e = E->dA.alloc(4 * n)) != cudaSuccess || (e = E->dM.alloc(2 * n)) != cudaSuccess ||
        (e = E->tiles.alloc(t.size())) != cudaSuccess) {
        E->release();
        delete E;
        return fail(e == cudaErrorMemoryAllocation ? MOHID_AD_ERR_ALLOC : MOHID_AD_ERR_CUDA, stat, cuda_msg("cudaMalloc", e));
    }
    if ((e = cudaMemcpy(E->tiles.p, t.data(), t.size() * sizeof(int4), cudaMemcpyHostToDevice)) != cudaSuccess) {
        E->release();
        delete E;
        return fail(MOHID_AD_ERR_CUDA, stat, cuda_msg("cudaMemcpy", e));
    }
    {
        std::lock_guard<std::mutex> lk(g_bmu);
        *eid = g_next_eid++;
        g_ens[*eid] = E;
        for (Batch* b : m) b->ensemble = *eid;
    }
    return ok(stat);
}

int mohid_ad_ensemble_step(const int* eid, const mohid_ad_params* p, const int* nsteps, const int* use_graph,
                           int* stat)
{
    TraceRange trace_("mohid_ad_ensemble_step");
    Ensemble* E = elookup(eid);
    if (!E) return fail(MOHID_AD_ERR_ID, stat, "unknown ensemble id");
    if (!p || !nsteps || !use_graph) return fail(MOHID_AD_ERR_NULLPTR, stat, "NULL argument");
    if (*nsteps < 1) return fail(MOHID_AD_ERR_BOUNDS, stat, "nsteps must be >= 1");
    const size_t n = E->m.size();
    const int method = p[0].AdvMethodH, limiter = p[0].TVDLimitationH;
    CK(cudaSetDevice(E->device));
    for (size_t q = 0; q < n; ++q) {
        Batch* b = E->m[q];
        b->fluxLast = false;
        std::string why;
        int code = check_batched_params(&p[q], b->hasRef, why, true);
        if (code) return fail(code, stat, "member " + std::to_string(q) + ": " + why);
        if (b->in->hasDisch)
            return fail(MOHID_AD_ERR_UNSUPPORTED, stat, "member " + std::to_string(q) +
                        ": ensembles without discharges (use a batch per domain)");
        b->dischOn = false;
        b->bcFix = bc_fixable(b, &p[q]);
        if (p[q].AdvMethodH != method || (method != MOHID_UPWIND_ORDER1 && p[q].TVDLimitationH != limiter))
            return fail(MOHID_AD_ERR_OPTION, stat, "members must share AdvMethodH and TVDLimitationH");
        if (b->hasRef)
            for (int t = 0; t < b->nt; ++t)
                if (t >= (int)b->refShift.size() || b->refShift[t] != b->shift[t])
                    return fail(MOHID_AD_ERR_OPTION, stat,
                                "set the reference of every tracer after (re)loading the tracer");
        {
            int c = ensure_packed(b, stat);
            if (c) return c;
        }
        int c = ensure_noflux(b, &p[q], stat);   // clears the bits of an earlier stand-alone step
        if (c) return c;
        c = ensure_shift_valid(b, &p[q], stat);
        if (c) return c;
        if (fix_active(b)) b->fixDirty = true;
        if (b->cur != E->cur) return fail(MOHID_AD_ERR_OPTION, stat, "a member was stepped outside the ensemble");
        if (b->sumsTh != -1 && b->sumsTh != 0)     // ensembles walk 8-row tiles
            CK(cudaMemsetAsync(b->mpart.p, 0, sizeof(double) * (size_t)b->nt * b->ntiles[1], b->in->stream));
        b->sumsTh = 0;
    }
    // members' own streams (packing, tracer loads) before the ensemble's
    for (size_t q = 0; q < n; ++q)
        if (E->m[q]->in->stream != E->s) CK(cudaStreamSynchronize(E->m[q]->in->stream));
    // argument tables for both buffer parities, without and with the fixer's
    // sums; tensor-map tables for both parities
    std::vector<mohid::BatchArgs> hA(4 * n);
    std::vector<mohid::TmaMaps> hM(2 * n);
    const int gi = E->nt == 4 ? 2 : (E->nt == 2 ? 1 : 0);
    for (int c = 0; c < 2; ++c)
        for (size_t q = 0; q < n; ++q) {
            Batch* b = E->m[q];
            const float* Pin = c ? b->PB.p : b->PA.p;
            float* Pout = c ? b->PA.p : b->PB.p;
            for (int l = 0; l < 2; ++l)
                hA[(c * 2 + l) * n + q] = make_bargs(b, &p[q], 0, b->nt, Pin, Pout, l == 1);
            hM[c * n + q] = b->maps[0];              // ensembles walk 8-row tiles
            hM[c * n + q].P = b->mapP[0][c][gi];
        }
    const bool same = E->uploaded && std::memcmp(hA.data(), E->hA.data(), hA.size() * sizeof(hA[0])) == 0 &&
                      std::memcmp(hM.data(), E->hM.data(), hM.size() * sizeof(hM[0])) == 0;
    if (!same) {
        CK(cudaStreamSynchronize(E->s));             // no launch still reads the tables
        CK(cudaMemcpy(E->dA.p, hA.data(), hA.size() * sizeof(hA[0]), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(E->dM.p, hM.data(), hM.size() * sizeof(hM[0]), cudaMemcpyHostToDevice));
        E->hA.swap(hA);
        E->hM.swap(hM);
        E->uploaded = true;
    }
    const int slots = mohid::ensemble_slots(E->nt, method, limiter, E->device);
    if (slots <= 0) return fail(MOHID_AD_ERR_CUDA, stat, "ensemble kernel occupancy query failed");
    const int grid = std::min(slots, E->ntiles);
    const bool cur0 = E->cur;
    auto flip_members = [&](int steps) {
        if (steps % 2)
            for (Batch* b : E->m) b->cur = !b->cur;
    };
    if (!*use_graph) {
        for (int q = 0; q < *nsteps; ++q) CK(enqueue_ens_step(E, method, limiter, grid, q == *nsteps - 1));
        flip_members(*nsteps);
        return ok(stat);
    }
    const int pairs = *nsteps / 2;
    if (pairs > 0) {
        const bool glast = *nsteps % 2 == 0;          // the graph holds the call's last step
        const bool reuse = E->graph && E->graphSteps == 2 * pairs && E->graphCur == E->cur &&
                           E->graphMethod == method && E->graphLimiter == limiter && E->graphLast == glast && same;
        if (!reuse) {
            if (E->graph) { cudaGraphExecDestroy(E->graph); E->graph = nullptr; }
            cudaGraph_t g;
            CK(cudaStreamBeginCapture(E->s, cudaStreamCaptureModeThreadLocal));
            cudaError_t e = cudaSuccess;
            for (int q = 0; q < 2 * pairs && e == cudaSuccess; ++q)
                e = enqueue_ens_step(E, method, limiter, grid, glast && q == 2 * pairs - 1);
            cudaError_t e2 = cudaStreamEndCapture(E->s, &g);
            E->cur = cur0;
            if (e != cudaSuccess) return fail(MOHID_AD_ERR_CUDA, stat, cuda_msg("capture", e));
            if (e2 != cudaSuccess) return fail(MOHID_AD_ERR_CUDA, stat, cuda_msg("cudaStreamEndCapture", e2));
            e = cudaGraphInstantiate(&E->graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) { E->graph = nullptr; return fail(MOHID_AD_ERR_CUDA, stat, cuda_msg("cudaGraphInstantiate", e)); }
            E->graphSteps = 2 * pairs;
            E->graphCur = cur0;
            E->graphMethod = method;
            E->graphLimiter = limiter;
            E->graphLast = glast;
        }
        CK(cudaGraphLaunch(E->graph, E->s));
    }
    if (*nsteps % 2) CK(enqueue_ens_step(E, method, limiter, grid, true));
    flip_members(*nsteps);
    return ok(stat);
}

int mohid_ad_ensemble_destroy(int* eid, int* stat)
{
    Ensemble* E = nullptr;
    if (eid) {
        std::lock_guard<std::mutex> lk(g_bmu);
        auto it = g_ens.find(*eid);
        if (it != g_ens.end()) {
            E = it->second;
            g_ens.erase(it);
            for (Batch* b : E->m) b->ensemble = 0;
        }
    }
    if (!E) return fail(MOHID_AD_ERR_ID, stat, "unknown ensemble id");
    cudaSetDevice(E->device);
    cudaStreamSynchronize(E->s);
    E->release();
    delete E;
    *eid = 0;
    return ok(stat);
}

}  // extern "C"
