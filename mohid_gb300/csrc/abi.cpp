// abi.cpp -- C-ABI of the GB300 advection-diffusion step (declared in include/mohid_ad.h).
//
// Host-side replacement for the reference's transport entry point and for the
// legacy CUDA Thomas binding:
//   AdvectionDiffusion        ModuleAdvectionDiffusion.F90:1108-1509
//   StartAdvectionDiffusion   ModuleAdvectionDiffusion.F90:400-535
//   KillAdvectionDiffusion    ModuleAdvectionDiffusion.F90:5849
//   SolveThomas_C & co.       Software/CudaThomas/Thomas.cu:6-56
// Instances live in a mutex-protected registry keyed by an int id (the legacy
// code used an unlocked static std::map, Thomas.cu:206).  Nothing here exits
// the process: every failure becomes a status code.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/mohid_ad.h"
#include "common.cuh"
#include "instance.hpp"

namespace mohid_abi {

thread_local std::string g_last_error = "";

int fail(int code, int* stat, const std::string& msg)
{
    g_last_error = msg;
    if (stat) *stat = code;
    return code;
}

int ok(int* stat)
{
    if (stat) *stat = MOHID_AD_SUCCESS;
    return MOHID_AD_SUCCESS;
}

int g_fail_alloc = 0;

void Instance::release()
{
    DevBuf<double>* d[] = {&DUX, &DVY, &DZX, &DZY, &Qx, &Qy, &Qz, &Vold, &V, &ViscH,
                           &DiffV, &AreaU, &AreaV, &DZZ, &DWZ, &Pin, &Pout, &Ref, &sys, &Wl, &Pmid, &flux,
                           &DUZ, &DVZ};
    for (auto* b : d) b->release();
    DevBuf<int>* i[] = {&KFloor, &BP2D, &OP, &LP, &WP, &CFU, &CFV, &CFW, &SD, &bcols, &cycl, &NFU, &NFV, &NFW,
                        &dStart};
    for (auto* b : i) b->release();
    dTerms.release();
    hasDisch = false;
    status.release();
    if (hstatus) cudaFreeHost(hstatus);
    hstatus = nullptr;
    if (stream) cudaStreamDestroy(stream);
    stream = nullptr;
}

std::mutex g_mu;
std::map<int, Instance*> g_inst;
int g_next_id = 1;

Instance* lookup(const int* id)
{
    if (!id) return nullptr;
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_inst.find(*id);
    return it == g_inst.end() ? nullptr : it->second;
}

std::string cuda_msg(const char* what, cudaError_t e)
{
    return std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
}


// Option checks of AdvectionDiffusion (AD:1231-1239, AD:1340-1349,
// Set_Internal_State AD:5816-5830) plus the options this library leaves out.
int check_params(const mohid_ad_params* p, bool hasRef, int nk, std::string& why)
{
    if (!p) { why = "params is NULL"; return MOHID_AD_ERR_NULLPTR; }
    if (!(p->DTProp > 0.0) || !std::isfinite(p->DTProp)) { why = "DTProp must be > 0"; return MOHID_AD_ERR_OPTION; }
    const int mH = p->AdvMethodH, mV = p->AdvMethodV;
    if (mH < 1 || mH > 6 || mV < 1 || mV > 6) { why = "AdvMethodH/V must be 1..6"; return MOHID_AD_ERR_OPTION; }
    if ((p->ImpExp_AdvXX == 1.0 || p->ImpExp_AdvYY == 1.0) && (mH == 2 || mH == 3)) {
        why = "implicit horizontal advection with UpwindOrder2/3 (reference ERR100)"; return MOHID_AD_ERR_OPTION;
    }
    if (p->ImpExp_AdvV == 1.0 && (mV == 2 || mV == 3)) {
        why = "implicit vertical advection with UpwindOrder2/3 (reference ERR200)"; return MOHID_AD_ERR_OPTION;
    }
    if (p->ImpExp_DifH != 0.0) { why = "horizontal diffusion must be explicit (reference ERR02)"; return MOHID_AD_ERR_OPTION; }
    if (p->ImpExp_AdvXX == 1.0 && p->ImpExp_AdvYY == 1.0) { why = "implicit advection in both horizontal directions (reference ERR03)"; return MOHID_AD_ERR_OPTION; }
    if (p->ImpExp_AdvV != 0.0 && p->ImpExp_AdvV != 1.0) { why = "ImpExp_AdvV must be 0 or 1 (reference ERR01)"; return MOHID_AD_ERR_OPTION; }
    if ((mH >= 2 && mH <= 4) && !p->Upwind2H) { why = "AdvMethodH 2..4 needs Upwind2H near boundaries"; return MOHID_AD_ERR_OPTION; }
    if ((mV >= 2 && mV <= 4) && !p->Upwind2V) { why = "AdvMethodV 2..4 needs Upwind2V near boundaries"; return MOHID_AD_ERR_OPTION; }
    if (mH == 4 && (p->TVDLimitationH < 1 || p->TVDLimitationH > 5)) { why = "TVDLimitationH must be 1..5"; return MOHID_AD_ERR_OPTION; }
    if (mV == 4 && (p->TVDLimitationV < 1 || p->TVDLimitationV > 5)) { why = "TVDLimitationV must be 1..5"; return MOHID_AD_ERR_OPTION; }
    if (p->Docycle_method != 1 && p->Docycle_method != 2) { why = "Docycle_method must be 1 or 2"; return MOHID_AD_ERR_OPTION; }
    {
        const int bc = p->BoundaryCondition;
        if (hasRef) {
            if (bc != 1 && bc != 2 && bc != 4 && bc != 5 && bc != 6 && bc != 7 && bc != 8) {
                why = "invalid BoundaryCondition (reference Set_Internal_State ERR01)"; return MOHID_AD_ERR_OPTION;
            }
        } else if (bc == MOHID_BC_CYCLIC) {
            why = "cyclic boundaries read ReferenceProp (reference Prop_CyclicBoundary)"; return MOHID_AD_ERR_OPTION;
        }
    }
    if ((p->ImpExp_AdvXX != 0.0 && p->ImpExp_AdvXX != 1.0) || (p->ImpExp_AdvYY != 0.0 && p->ImpExp_AdvYY != 1.0)) {
        why = "ImpExp_AdvXX / ImpExp_AdvYY must be 0 or 1 (reference HorizontalAdvectionXX/YY ERR01)";
        return MOHID_AD_ERR_OPTION;
    }
    if (p->AdvectionNudging && (p->ImpExp_AdvXX != 0.0 || p->ImpExp_AdvYY != 0.0 || p->Vertical1D)) {
        // the _Nudge routines put implicit horizontal coefficients into the
        // vertical system (AD:4692-4696), and with Vertical1D AdvectionNudging
        // reads arrays nothing set in the call (AD:1704, AD:4151-4157)
        why = "AdvectionNudging with implicit horizontal advection or Vertical1D";
        return MOHID_AD_ERR_UNSUPPORTED;
    }
    if (nk > 200) { why = "KUB > 200 layers not supported"; return MOHID_AD_ERR_UNSUPPORTED; }
    return MOHID_AD_SUCCESS;
}

int status_to_code(unsigned int s, std::string& why)
{
    if (s & MOHID_DEV_BAD_FACE) { why = "a compute face lies on the lower edge of the work box"; return MOHID_AD_ERR_BOUNDS; }
    if (s & MOHID_DEV_ZERO_PIVOT) { why = "THOMASZ zero pivot in a water column"; return MOHID_AD_ERR_ZERO_PIVOT; }
    if (s & MOHID_DEV_NONFINITE) { why = "non-finite concentration after the solve"; return MOHID_AD_ERR_NONFINITE; }
    if (s & MOHID_DEV_TIMEOUT) { why = "bounded device wait expired"; return MOHID_AD_ERR_TIMEOUT; }
    if (s & MOHID_DEV_OBC_EDGE) {
        why = "Orlanski: an open boundary point off the work box's edges (reference 'Orlanski Advection 2')";
        return MOHID_AD_ERR_OPTION;
    }
    if (s & MOHID_DEV_OBC_READ) { why = "Orlanski: a read outside the layer plane (grid under 3 cells wide)"; return MOHID_AD_ERR_BOUNDS; }
    return MOHID_AD_SUCCESS;
}

mohid::PlainArgs make_args(Instance* in, const double* Pin, double* Pout, const double* Ref,
                           const mohid_ad_params* p);

// One step of one property, P_in -> P_out (device, Size box), on the
// instance's stream.  Implicit horizontal advection (AD:4167-4254,
// AD:1758-1858): in 3-D the rows of the horizontal system, its line solve into
// Pmid, then the column step from Pmid; with one layer the rows (open
// boundaries and land included) and the line solve instead of the columns.
cudaError_t post_solve(Instance* in, double* P, const double* Ref, const mohid_ad_params* p);

// One step of one property, P_in -> P_out (device, Size box), on the
// instance's stream: the solve (below), the boundary conditions applied after
// it, and with CellFluxes the face fluxes (zeroed first, explicit parts
// recorded by the step, implicit parts added after the solve, AD:1458-1468,
// AD:1882-1916).  Implicit horizontal advection (AD:4167-4254, AD:1758-1858):
// in 3-D the rows of the horizontal system, its line solve into Pmid, then the
// column step from Pmid; with one layer the rows (open boundaries and land
// included) and the line solve instead of the columns.
int run_step(Instance* in, const double* Pin, double* Pout, const double* Ref, const mohid_ad_params* p,
             int* stat)
{
    cudaStream_t s = in->stream;
    if ((p->NoAdvFlux || p->NoDifFlux) && !in->hasNoFlux)
        return fail(MOHID_AD_ERR_NULLPTR, stat, "NoAdvFlux / NoDifFlux need the NoFluxU/V/W masks (mohid_ad_set_noflux)");
    const bool cflux = p->CellFluxes != 0;
    auto bad_alloc = [&](cudaError_t e) {
        return fail(e == cudaErrorMemoryAllocation ? MOHID_AD_ERR_ALLOC : MOHID_AD_ERR_CUDA, stat,
                    cuda_msg("cudaMalloc", e));
    };
    in->fluxLast = false;
    if (cflux) {
        if (!in->flux.p) {
            cudaError_t e = in->flux.alloc(6 * in->n3);
            if (e != cudaSuccess) { in->flux.release(); return bad_alloc(e); }
        }
        CK(cudaMemsetAsync(in->flux.p, 0, sizeof(double) * 6 * in->n3, s));
    }
    auto args = [&](const double* Pi, double* Po) {
        mohid::PlainArgs x = make_args(in, Pi, Po, Ref, p);
        if (cflux) {
            double* f = in->flux.p;
            x.fAX = f; x.fAY = f + in->n3; x.fAZ = f + 2 * in->n3;
            x.fDX = f + 3 * in->n3; x.fDY = f + 4 * in->n3; x.fDZ = f + 5 * in->n3;
        }
        return x;
    };
    // Orlanski boundaries: the caller's PropOld and the radiated exterior
    // values of the field the boundary condition sees (AD:5428-5429, 5496-5569)
    const bool orl = Ref && p->BoundaryCondition == MOHID_BC_ORLANSKI;
    const size_t bd = sizeof(double) * in->n3;
    if (orl && !in->Pobc.p) {
        cudaError_t e = in->Pobc.alloc(in->n3);
        if (e != cudaSuccess) { in->Pobc.release(); return bad_alloc(e); }
    }
    auto orlanski = [&](mohid::PlainArgs& x) -> cudaError_t {
        if (!orl) return cudaSuccess;
        cudaError_t e = cudaMemcpyAsync(in->Pobc.p, x.P, bd, cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess && in->propOld)
            e = cudaMemcpyAsync(in->propOld, x.P, bd, in->propOldDev ? cudaMemcpyDeviceToDevice
                                                                      : cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = mohid::launch_orlanski(x, in->Pobc.p, in->bcols.p, in->nbcols, s);
        x.Pobc = in->Pobc.p;
        return e;
    };
    mohid::PlainArgs a = args(Pin, Pout);
    const bool imp = a.impXX || a.impYY;
    const bool lines3D = imp && in->nk > 1 && !a.vertical1D;
    const bool lines2D = imp && in->nk == 1;
    mohid::PlainArgs v = a;                      // the field the vertical terms see
    if (!lines3D && !lines2D) {
        CK(orlanski(a));
        CK(mohid::launch_plain_f64(a, s));
    } else {
        if (!in->sys.p) {
            cudaError_t e = in->sys.alloc(4 * in->n3);
            if (e == cudaSuccess) e = in->Wl.alloc(in->n3);
            if (e == cudaSuccess) e = in->Pmid.alloc(in->n3);
            if (e != cudaSuccess) { in->sys.release(); in->Wl.release(); in->Pmid.release(); return bad_alloc(e); }
        }
        a.sD = in->sys.p; a.sE = a.sD + in->n3; a.sF = a.sE + in->n3; a.sTI = a.sF + in->n3;
        if (lines3D) {
            CK(mohid::launch_plain_f64(a, s, mohid::kPlainHorizRows));
            CK(cudaMemcpyAsync(in->Pmid.p, Pin, bd, cudaMemcpyDeviceToDevice, s));
            CK(mohid::launch_line_solve(in->ni, in->nj, in->nk, a.impXX != 0, a.sD, a.sE, a.sF, a.sTI, in->LP.p,
                                        false, in->Wl.p, in->Pmid.p, in->status.p, s));
            v = args(in->Pmid.p, Pout);
            CK(orlanski(v));
            CK(mohid::launch_plain_f64(v, s, mohid::kPlainVertical));
        } else {
            CK(orlanski(a));
            CK(mohid::launch_plain_f64(a, s, mohid::kPlainRows2D));
            CK(cudaMemcpyAsync(Pout, orl ? in->Pobc.p : Pin, bd, cudaMemcpyDeviceToDevice, s));
            CK(mohid::launch_line_solve(in->ni, in->nj, in->nk, a.impXX != 0, a.sD, a.sE, a.sF, a.sTI, in->LP.p,
                                        true, in->Wl.p, Pout, in->status.p, s));
        }
    }
    CK(post_solve(in, Pout, Ref, p));
    if (cflux) {
        CK(mohid::launch_cell_fluxes(a, v, Pout, p->ImpExp_AdvV, p->ImpExp_DifV, s));
        in->fluxLast = true;
    }
    return ok(stat);
}

// boundary conditions the reference applies after the solve (AD:1874-1880),
// whether or not a reference is given
cudaError_t post_solve(Instance* in, double* P, const double* Ref, const mohid_ad_params* p)
{
    if (p->BoundaryCondition == MOHID_BC_NULL_GRADIENT)
        return mohid::launch_null_gradient(in->ni, in->nj, in->nk, P, in->CFU.p, in->CFV.p, in->KFloor.p,
                                           in->bcols.p, in->nbcols, in->stream);
    if (p->BoundaryCondition == MOHID_BC_CYCLIC)
        return mohid::launch_cyclic(in->ni, in->nj, in->nk, P, Ref, in->KFloor.p, in->bcols.p, in->nbcols,
                                    in->cycl.p, in->nrows, in->ncyc, in->stream);
    return cudaSuccess;
}

mohid::PlainArgs make_args(Instance* in, const double* Pin, double* Pout, const double* Ref,
                           const mohid_ad_params* p)
{
    mohid::PlainArgs a;
    a.ni = in->ni; a.nj = in->nj; a.nk = in->nk;
    a.sj = in->ni + 2;
    a.sk = (long long)(in->ni + 2) * (in->nj + 2);
    a.P = Pin; a.Pout = Pout;
    a.Qx = in->Qx.p; a.Qy = in->Qy.p; a.Qz = in->Qz.p; a.Vold = in->Vold.p; a.V = in->V.p;
    a.ViscH = in->ViscH.p; a.DiffV = in->DiffV.p; a.AreaU = in->AreaU.p; a.AreaV = in->AreaV.p;
    a.DZZ = in->DZZ.p; a.DWZ = in->DWZ.p;
    a.OP = in->OP.p; a.LP = in->LP.p; a.WP = in->WP.p; a.CFU = in->CFU.p; a.CFV = in->CFV.p;
    a.CFW = in->CFW.p; a.SD = in->hasSD ? in->SD.p : nullptr;
    a.DUX = in->DUX.p; a.DVY = in->DVY.p; a.DZX = in->DZX.p; a.DZY = in->DZY.p;
    a.KFloor = in->KFloor.p; a.BP2D = in->BP2D.p;
    a.Ref = Ref;
    a.Pobc = nullptr;
    a.DT = p->DTProp;
    a.schmidtH = p->schmidt_H; a.schmidtCoefV = p->SchmidtCoef_V; a.schmidtBackV = p->SchmidtBackground_V;
    a.volumeRelMax = p->VolumeRelMax; a.impExpDifV = p->ImpExp_DifV;
    // OpenBoundaryCondition AD:5418-5419: TdecAux = 1/(1 + DecayTime/DTProp)
    a.tdecAux = 1.0 / (1.0 + p->DecayTime / p->DTProp);
    a.methodH = p->AdvMethodH; a.limiterH = p->TVDLimitationH;
    a.methodV = p->AdvMethodV; a.limiterV = p->TVDLimitationV;
    a.upwind2H = p->Upwind2H != 0; a.upwind2V = p->Upwind2V != 0;
    a.nullDif = p->NullDif != 0;
    a.explicitV = p->ImpExp_AdvV == 0.0;
    a.docycle = p->Docycle_method;
    a.vertical1D = p->Vertical1D != 0; a.xzflow = p->XZFlow != 0;
    a.bc = p->BoundaryCondition;
    a.impXX = p->ImpExp_AdvXX == 1.0;
    a.impYY = p->ImpExp_AdvYY == 1.0;
    a.sD = a.sE = a.sF = a.sTI = nullptr;
    a.fAX = a.fAY = a.fAZ = a.fDX = a.fDY = a.fDZ = nullptr;
    a.nudge = p->AdvectionNudging != 0;
    a.nudgeCells = p->AdvectionNudgingCells;
    a.noAdv = p->NoAdvFlux != 0 && !a.nudge;     // the _Nudge routines ignore the NoAdvFlux masks
    a.noDif = p->NoDifFlux != 0;
    a.NFU = in->hasNoFlux ? in->NFU.p : nullptr;
    a.NFV = in->hasNoFlux ? in->NFV.p : nullptr;
    a.NFW = in->hasNoFlux ? in->NFW.p : nullptr;
    a.dStart = in->hasDisch ? in->dStart.p : nullptr;
    a.dTerms = in->hasDisch ? in->dTerms.p : nullptr;
    a.status = in->status.p;
    return a;
}

// fromDevice: device arrays; bind: the FP64 device arrays are borrowed in
// place (read, and written by the device producers) instead of copied
int upload_hydro(Instance* in, bool fromDevice, bool bind, const double* Wflux_X, const double* Wflux_Y,
                 const double* Wflux_Z, const double* VolumeZOld, const double* VolumeZ,
                 const double* Visc_H, const double* Diff_V, const double* AreaU,
                 const double* AreaV, const double* DZZ, const double* DWZ, const int* OpenPoints3D,
                 const int* LandPoints3D, const int* WaterPoints3D, const int* ComputeFacesU3D,
                 const int* ComputeFacesV3D, const int* ComputeFacesW3D, const int* SmallDepths,
                 int* stat)
{
    const double* ds[] = {Wflux_X, Wflux_Y, Wflux_Z, VolumeZOld, VolumeZ, Visc_H, Diff_V, AreaU, AreaV, DZZ, DWZ};
    const int* is[] = {OpenPoints3D, LandPoints3D, WaterPoints3D, ComputeFacesU3D, ComputeFacesV3D, ComputeFacesW3D};
    // After the first complete call, a NULL array keeps the instance's copy
    // (unchanged since the last call, or produced on the device); the six
    // masks are given all together or not at all.
    int nmask = 0;
    for (const int* m : is) nmask += m != nullptr;
    if (!in->hydro) {
        for (const double* d : ds)
            if (!d) return fail(MOHID_AD_ERR_NULLPTR, stat, "a required hydrodynamic array is NULL");
        if (nmask != 6) return fail(MOHID_AD_ERR_NULLPTR, stat, "a required mask array is NULL");
    } else if (nmask != 0 && nmask != 6) {
        return fail(MOHID_AD_ERR_NULLPTR, stat, "give the six 3-D masks together, or none to keep them");
    }
    const cudaMemcpyKind kind = fromDevice ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    CK(cudaSetDevice(in->device));
    const size_t bd = sizeof(double) * in->n3, bi = sizeof(int) * in->n3;
    DevBuf<double>* dd[] = {&in->Qx, &in->Qy, &in->Qz, &in->Vold, &in->V, &in->ViscH, &in->DiffV,
                            &in->AreaU, &in->AreaV, &in->DZZ, &in->DWZ};
    for (int q = 0; q < 11; ++q) {
        if (!ds[q]) continue;
        if (bind) {
            dd[q]->borrow(const_cast<double*>(ds[q]));
        } else {
            dd[q]->unborrow();
            CK(cudaMemcpyAsync(dd[q]->p, ds[q], bd, kind, in->stream));
        }
    }
    ++in->hydroVersion;
    if (nmask == 0) {
        // the masks stay; host buffers are consumed before returning
        if (!fromDevice) CK(cudaStreamSynchronize(in->stream));
        return ok(stat);
    }
    DevBuf<int>* di[] = {&in->OP, &in->LP, &in->WP, &in->CFU, &in->CFV, &in->CFW};
    for (int q = 0; q < 6; ++q) CK(cudaMemcpyAsync(di[q]->p, is[q], bi, kind, in->stream));
    in->hasSD = SmallDepths != nullptr;
    if (SmallDepths) CK(cudaMemcpyAsync(in->SD.p, SmallDepths, sizeof(int) * in->n2, kind, in->stream));
    ++in->maskVersion;
    CK(cudaMemsetAsync(in->status.p, 0, sizeof(unsigned int), in->stream));
    CK(mohid::launch_check_faces(in->ni, in->nj, in->nk, in->CFU.p, in->CFV.p, in->CFW.p,
                                 in->status.p, in->stream));
    CK(cudaMemcpyAsync(in->hstatus, in->status.p, sizeof(unsigned int), cudaMemcpyDeviceToHost, in->stream));
    CK(cudaStreamSynchronize(in->stream));
    std::string why;
    int code = status_to_code(*in->hstatus, why);
    in->hydro = code == MOHID_AD_SUCCESS;
    if (code) return fail(code, stat, why);
    return ok(stat);
}

}  // namespace mohid_abi

using namespace mohid_abi;

extern "C" {

void mohid_ad_default_params(mohid_ad_params* p)
{
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->schmidt_H = 1.0;
    p->SchmidtCoef_V = 1.0;
    p->SchmidtBackground_V = 1e-8;
    p->AdvMethodH = MOHID_UPWIND_ORDER1;
    p->TVDLimitationH = MOHID_TVD_SUPERBEE;
    p->AdvMethodV = MOHID_UPWIND_ORDER1;
    p->TVDLimitationV = MOHID_TVD_SUPERBEE;
    p->VolumeRelMax = 1.5;
    p->DTProp = 1.0;
    p->ImpExp_AdvV = 1.0;
    p->ImpExp_DifV = 1.0;
    p->BoundaryCondition = MOHID_BC_MASS_CONSERVATION;
    p->DecayTime = 0.0;
    p->Docycle_method = 1;
}

const char* mohid_ad_last_error(void) { return g_last_error.c_str(); }

const char* mohid_ad_version(void) { return "mohid-gb300 0.1 sm_103a"; }

int mohid_ad_init(int* id, const T_Size3D* size, const T_Size3D* worksize, const double* DUX,
                  const double* DVY, const double* DZX, const double* DZY, const int* KFloorZ,
                  const int* BoundaryPoints2D, int* stat)
{
    TraceRange trace_("mohid_ad_init");
    if (!id || !size || !worksize || !DUX || !DVY || !DZX || !DZY || !KFloorZ || !BoundaryPoints2D)
        return fail(MOHID_AD_ERR_NULLPTR, stat, "mohid_ad_init: NULL argument");
    const T_Size3D& s = *size;
    const T_Size3D& w = *worksize;
    if (w.ILB != 1 || w.JLB != 1 || w.KLB != 1 || w.IUB < 1 || w.JUB < 1 || w.KUB < 1 ||
        s.ILB != w.ILB - 1 || s.IUB != w.IUB + 1 || s.JLB != w.JLB - 1 || s.JUB != w.JUB + 1 ||
        s.KLB != w.KLB - 1 || s.KUB != w.KUB + 1)
        return fail(MOHID_AD_ERR_BOUNDS, stat,
                    "mohid_ad_init: WorkSize must start at 1 and Size must be WorkSize +/- 1");
    Instance* in = new Instance();
    in->ni = w.IUB; in->nj = w.JUB; in->nk = w.KUB;
    in->n2 = (size_t)(in->ni + 2) * (size_t)(in->nj + 2);
    in->n3 = in->n2 * (size_t)(in->nk + 2);
    auto bad = [&](cudaError_t e, const char* what) {
        std::string m = cuda_msg(what, e);
        in->release();
        delete in;
        int code = (e == cudaErrorMemoryAllocation) ? MOHID_AD_ERR_ALLOC : MOHID_AD_ERR_CUDA;
        return fail(code, stat, m);
    };
    cudaError_t e = cudaGetDevice(&in->device);
    if (e != cudaSuccess) return bad(e, "cudaGetDevice");
    if ((e = cudaStreamCreateWithFlags(&in->stream, cudaStreamNonBlocking)) != cudaSuccess) return bad(e, "cudaStreamCreate");
    DevBuf<double>* d2[] = {&in->DUX, &in->DVY, &in->DZX, &in->DZY};
    for (auto* b : d2) if ((e = b->alloc(in->n2)) != cudaSuccess) return bad(e, "cudaMalloc");
    DevBuf<int>* i2[] = {&in->KFloor, &in->BP2D, &in->SD};
    for (auto* b : i2) if ((e = b->alloc(in->n2)) != cudaSuccess) return bad(e, "cudaMalloc");
    DevBuf<double>* d3[] = {&in->Qx, &in->Qy, &in->Qz, &in->Vold, &in->V, &in->ViscH, &in->DiffV,
                            &in->AreaU, &in->AreaV, &in->DZZ, &in->DWZ, &in->Pin, &in->Pout, &in->Ref};
    for (auto* b : d3) if ((e = b->alloc(in->n3)) != cudaSuccess) return bad(e, "cudaMalloc");
    DevBuf<int>* i3[] = {&in->OP, &in->LP, &in->WP, &in->CFU, &in->CFV, &in->CFW};
    for (auto* b : i3) if ((e = b->alloc(in->n3)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = in->status.alloc(1)) != cudaSuccess) return bad(e, "cudaMalloc");
    if ((e = cudaMallocHost((void**)&in->hstatus, sizeof(unsigned int))) != cudaSuccess) return bad(e, "cudaMallocHost");
    const double* s2[] = {DUX, DVY, DZX, DZY};
    for (int q = 0; q < 4; ++q)
        if ((e = cudaMemcpy(d2[q]->p, s2[q], sizeof(double) * in->n2, cudaMemcpyHostToDevice)) != cudaSuccess)
            return bad(e, "cudaMemcpy");
    if ((e = cudaMemcpy(in->KFloor.p, KFloorZ, sizeof(int) * in->n2, cudaMemcpyHostToDevice)) != cudaSuccess) return bad(e, "cudaMemcpy");
    in->hKFloor.assign(KFloorZ, KFloorZ + in->n2);
    if ((e = cudaMemcpy(in->BP2D.p, BoundaryPoints2D, sizeof(int) * in->n2, cudaMemcpyHostToDevice)) != cudaSuccess) return bad(e, "cudaMemcpy");
    {
        // boundary columns in the reference's sweep order (j outer, i inner);
        // rows i with boundary points at j = 1 and nj, columns j with boundary
        // points at i = 1 and ni (Prop_CyclicBoundary AD:2171-2220)
        std::vector<int> cols, rows, cyc;
        const int ni = in->ni, nj = in->nj, sj = ni + 2;
        auto bp = [&](int i, int j) { return BoundaryPoints2D[(size_t)i + (size_t)sj * j] == 1; };
        for (int j = 1; j <= nj; ++j)
            for (int i = 1; i <= ni; ++i)
                if (bp(i, j)) cols.push_back(i + sj * j);
        for (int i = 2; i <= ni - 1; ++i)
            if (bp(i, 1) && bp(i, nj)) rows.push_back(i);
        for (int j = 2; j <= nj - 1; ++j)
            if (bp(1, j) && bp(ni, j)) cyc.push_back(j);
        in->nbcols = (int)cols.size();
        in->nrows = (int)rows.size();
        in->ncyc = (int)cyc.size();
        rows.insert(rows.end(), cyc.begin(), cyc.end());
        if ((e = in->bcols.alloc(cols.size())) != cudaSuccess) return bad(e, "cudaMalloc");
        if ((e = in->cycl.alloc(rows.size())) != cudaSuccess) return bad(e, "cudaMalloc");
        if (!cols.empty() && (e = cudaMemcpy(in->bcols.p, cols.data(), sizeof(int) * cols.size(),
                                             cudaMemcpyHostToDevice)) != cudaSuccess) return bad(e, "cudaMemcpy");
        if (!rows.empty() && (e = cudaMemcpy(in->cycl.p, rows.data(), sizeof(int) * rows.size(),
                                             cudaMemcpyHostToDevice)) != cudaSuccess) return bad(e, "cudaMemcpy");
    }
    {
        std::lock_guard<std::mutex> lk(g_mu);
        *id = g_next_id++;
        g_inst[*id] = in;
    }
    return ok(stat);
}

int mohid_ad_set_hydro(const int* id, const double* Wflux_X, const double* Wflux_Y,
                       const double* Wflux_Z, const double* VolumeZOld, const double* VolumeZ,
                       const double* Visc_H, const double* Diff_V, const double* AreaU,
                       const double* AreaV, const double* DZZ, const double* DWZ,
                       const int* OpenPoints3D, const int* LandPoints3D, const int* WaterPoints3D,
                       const int* ComputeFacesU3D, const int* ComputeFacesV3D,
                       const int* ComputeFacesW3D, const int* SmallDepths, int* stat)
{
    TraceRange trace_("mohid_ad_set_hydro");
    Instance* in = lookup(id);
    if (!in) return fail(MOHID_AD_ERR_ID, stat, "unknown instance id");
    return upload_hydro(in, false, false, Wflux_X, Wflux_Y, Wflux_Z, VolumeZOld, VolumeZ, Visc_H, Diff_V,
                        AreaU, AreaV, DZZ, DWZ, OpenPoints3D, LandPoints3D, WaterPoints3D,
                        ComputeFacesU3D, ComputeFacesV3D, ComputeFacesW3D, SmallDepths, stat);
}

int mohid_ad_set_hydro_dev(const int* id, const double* Wflux_X, const double* Wflux_Y,
                           const double* Wflux_Z, const double* VolumeZOld, const double* VolumeZ,
                           const double* Visc_H, const double* Diff_V, const double* AreaU,
                           const double* AreaV, const double* DZZ, const double* DWZ,
                           const int* OpenPoints3D, const int* LandPoints3D,
                           const int* WaterPoints3D, const int* ComputeFacesU3D,
                           const int* ComputeFacesV3D, const int* ComputeFacesW3D,
                           const int* SmallDepths, int* stat)
{
    TraceRange trace_("mohid_ad_set_hydro_dev");
    Instance* in = lookup(id);
    if (!in) return fail(MOHID_AD_ERR_ID, stat, "unknown instance id");
    return upload_hydro(in, true, false, Wflux_X, Wflux_Y, Wflux_Z, VolumeZOld, VolumeZ, Visc_H, Diff_V,
                        AreaU, AreaV, DZZ, DWZ, OpenPoints3D, LandPoints3D, WaterPoints3D,
                        ComputeFacesU3D, ComputeFacesV3D, ComputeFacesW3D, SmallDepths, stat);
}

int mohid_ad_bind_hydro_dev(const int* id, const double* Wflux_X, const double* Wflux_Y,
                            const double* Wflux_Z, const double* VolumeZOld, const double* VolumeZ,
                            const double* Visc_H, const double* Diff_V, const double* AreaU,
                            const double* AreaV, const double* DZZ, const double* DWZ,
                            const int* OpenPoints3D, const int* LandPoints3D,
                            const int* WaterPoints3D, const int* ComputeFacesU3D,
                            const int* ComputeFacesV3D, const int* ComputeFacesW3D,
                            const int* SmallDepths, int* stat)
{
    TraceRange trace_("mohid_ad_bind_hydro_dev");
    Instance* in = lookup(id);
    if (!in) return fail(MOHID_AD_ERR_ID, stat, "unknown instance id");
    return upload_hydro(in, true, true, Wflux_X, Wflux_Y, Wflux_Z, VolumeZOld, VolumeZ, Visc_H, Diff_V,
                        AreaU, AreaV, DZZ, DWZ, OpenPoints3D, LandPoints3D, WaterPoints3D,
                        ComputeFacesU3D, ComputeFacesV3D, ComputeFacesW3D, SmallDepths, stat);
}

int mohid_ad_get_hydro(const int* id, double* Wflux_X, double* Wflux_Y, double* Wflux_Z, double* VolumeZOld,
                       double* VolumeZ, double* Visc_H, double* Diff_V, double* AreaU, double* AreaV, double* DZZ,
                       double* DWZ, const int* on_device, int* stat)
{
    TraceRange trace_("mohid_ad_get_hydro");
    Instance* in = lookup(id);
    if (!in) return fail(MOHID_AD_ERR_ID, stat, "unknown instance id");
    if (!on_device) return fail(MOHID_AD_ERR_NULLPTR, stat, "NULL argument");
    if (!in->hydro) return fail(MOHID_AD_ERR_OPTION, stat, "the instance has no hydrodynamics set");
    CK(cudaSetDevice(in->device));
    double* dst[] = {Wflux_X, Wflux_Y, Wflux_Z, VolumeZOld, VolumeZ, Visc_H, Diff_V, AreaU, AreaV, DZZ, DWZ};
    DevBuf<double>* src[] = {&in->Qx, &in->Qy, &in->Qz, &in->Vold, &in->V, &in->ViscH, &in->DiffV,
                             &in->AreaU, &in->AreaV, &in->DZZ, &in->DWZ};
    const cudaMemcpyKind kind = *on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    for (int q = 0; q < 11; ++q)
        if (dst[q]) CK(cudaMemcpyAsync(dst[q], src[q]->p, sizeof(double) * in->n3, kind, in->stream));
    CK(cudaStreamSynchronize(in->stream));
    return ok(stat);
}

int mohid_ad_step_prop_f64_dev(const int* id, const double* PROP_in, double* PROP_out,
                               const double* ReferenceProp, const mohid_ad_params* p, int* stat)
{
    TraceRange trace_("mohid_ad_step_prop_f64_dev");
    Instance* in = lookup(id);
    if (!in) return fail(MOHID_AD_ERR_ID, stat, "unknown instance id");
    if (!PROP_in || !PROP_out) return fail(MOHID_AD_ERR_NULLPTR, stat, "PROP pointer is NULL");
    if (PROP_in == PROP_out) return fail(MOHID_AD_ERR_OPTION, stat, "PROP_in and PROP_out must differ");
    if (!in->hydro) return fail(MOHID_AD_ERR_OPTION, stat, "no hydrodynamics set for this instance");
    std::string why;
    int code = check_params(p, ReferenceProp != nullptr, in->nk, why);
    if (code) return fail(code, stat, why);
    CK(cudaSetDevice(in->device));
    return run_step(in, PROP_in, PROP_out, ReferenceProp, p, stat);
}

int mohid_ad_step_prop_f64(const int* id, double* PROP, const double* ReferenceProp,
                           const mohid_ad_params* p, int* stat)
{
    TraceRange trace_("mohid_ad_step_prop_f64");
    Instance* in = lookup(id);
    if (!in) return fail(MOHID_AD_ERR_ID, stat, "unknown instance id");
    if (!PROP) return fail(MOHID_AD_ERR_NULLPTR, stat, "PROP is NULL");
    if (!in->hydro) return fail(MOHID_AD_ERR_OPTION, stat, "no hydrodynamics set for this instance");
    std::string why;
    int code = check_params(p, ReferenceProp != nullptr, in->nk, why);
    if (code) return fail(code, stat, why);
    CK(cudaSetDevice(in->device));
    const size_t bd = sizeof(double) * in->n3;
    CK(cudaMemcpyAsync(in->Pin.p, PROP, bd, cudaMemcpyHostToDevice, in->stream));
    if (ReferenceProp) CK(cudaMemcpyAsync(in->Ref.p, ReferenceProp, bd, cudaMemcpyHostToDevice, in->stream));
    CK(cudaMemsetAsync(in->status.p, 0, sizeof(unsigned int), in->stream));
    code = run_step(in, in->Pin.p, in->Pout.p, ReferenceProp ? in->Ref.p : nullptr, p, stat);
    if (code) return code;
    CK(cudaMemcpyAsync(in->hstatus, in->status.p, sizeof(unsigned int), cudaMemcpyDeviceToHost, in->stream));
    CK(cudaMemcpyAsync(PROP, in->Pout.p, bd, cudaMemcpyDeviceToHost, in->stream));
    CK(cudaStreamSynchronize(in->stream));
    code = status_to_code(*in->hstatus, why);
    if (code) return fail(code, stat, why);
    return ok(stat);
}

int mohid_ad_step_f64(const int* id, double* PROP, const mohid_ad_params* p, const double* Wflux_X,
                      const double* Wflux_Y, const double* Wflux_Z, const double* VolumeZOld,
                      const double* VolumeZ, const double* Visc_H, const double* Diff_V,
                      const double* AreaU, const double* AreaV, const double* DZZ,
                      const double* DWZ, const int* OpenPoints3D, const int* LandPoints3D,
                      const int* WaterPoints3D, const int* ComputeFacesU3D,
                      const int* ComputeFacesV3D, const int* ComputeFacesW3D,
                      const int* SmallDepths, const double* ReferenceProp, int* stat)
{
    TraceRange trace_("mohid_ad_step_f64");
    int code = mohid_ad_set_hydro(id, Wflux_X, Wflux_Y, Wflux_Z, VolumeZOld, VolumeZ, Visc_H,
                                  Diff_V, AreaU, AreaV, DZZ, DWZ, OpenPoints3D, LandPoints3D,
                                  WaterPoints3D, ComputeFacesU3D, ComputeFacesV3D,
                                  ComputeFacesW3D, SmallDepths, stat);
    if (code) return code;
    return mohid_ad_step_prop_f64(id, PROP, ReferenceProp, p, stat);
}

int mohid_ad_sync(const int* id, int* stat)
{
    TraceRange trace_("mohid_ad_sync");
    Instance* in = lookup(id);
    if (!in) return fail(MOHID_AD_ERR_ID, stat, "unknown instance id");
    CK(cudaSetDevice(in->device));
    CK(cudaMemcpyAsync(in->hstatus, in->status.p, sizeof(unsigned int), cudaMemcpyDeviceToHost, in->stream));
    CK(cudaStreamSynchronize(in->stream));
    std::string why;
    int code = status_to_code(*in->hstatus, why);
    CK(cudaMemsetAsync(in->status.p, 0, sizeof(unsigned int), in->stream));
    if (code) return fail(code, stat, why);
    return ok(stat);
}

void* mohid_ad_stream(const int* id)
{
    Instance* in = lookup(id);
    return in ? (void*)in->stream : nullptr;
}

int mohid_ad_set_discharges(const int* id, const int* DischNumber, const int* DischnCells, const int* IgnoreDisch,
                            const int* ByPass, const int* DischVert, const int* DischI, const int* DischJ,
                            const int* DischK, const int* DischKmin, const int* DischKmax, const double* DischFlow,
                            const double* DischConc, const double* DischConcMF, int* stat)
{
    TraceRange trace_("mohid_ad_set_discharges");
    Instance* in = lookup(id);
    if (!in) return fail(MOHID_AD_ERR_ID, stat, "unknown instance id");
    if (!DischNumber) return fail(MOHID_AD_ERR_NULLPTR, stat, "NULL argument");
    const int nd = *DischNumber;
    if (nd < 0) return fail(MOHID_AD_ERR_BOUNDS, stat, "DischNumber must be >= 0");
    if (nd > 0 && (!DischnCells || !IgnoreDisch || !ByPass || !DischVert))
        return fail(MOHID_AD_ERR_NULLPTR, stat, "NULL argument");
    // the terms in the reference's order (AD:4040-4125): discharges not
    // ignored, their cells, the layers of each cell
    const int fillInt = -9999999, uniformVert = 5;   // FillValueInt, DischUniform_
    const int ni = in->ni, nj = in->nj, nk = in->nk, sj = ni + 2;
    struct Term { int col; mohid::DischTerm t; int cell; };   // column, term, discharge cell n
    std::vector<Term> terms;
    int n = 0;
    for (int dis = 0; dis < nd; ++dis) {
        if (IgnoreDisch[dis]) continue;
        if (DischnCells[dis] < 0) return fail(MOHID_AD_ERR_BOUNDS, stat, "DischnCells must be >= 0");
        const bool uniform = DischVert[dis] == uniformVert;
        for (int nc = 0; nc < DischnCells[dis]; ++nc, ++n) {
            if (!DischI || !DischJ || !DischK || !DischKmin || !DischKmax || !DischFlow || !DischConc || !DischConcMF)
                return fail(MOHID_AD_ERR_NULLPTR, stat, "NULL argument");
            const int i = DischI[n], j = DischJ[n];
            if (i < 1 || i > ni || j < 1 || j > nj) return fail(MOHID_AD_ERR_BOUNDS, stat, "discharge cell outside the work box");
            int kmin, kmax;
            if (uniform) {
                kmin = DischKmin[n] == fillInt ? in->hKFloor[(size_t)i + (size_t)sj * j] : DischKmin[n];
                kmax = DischKmax[n] == fillInt ? nk : DischKmax[n];
            } else {
                kmin = kmax = DischK[n];
            }
            if (kmin < 1 || kmax > nk) return fail(MOHID_AD_ERR_BOUNDS, stat, "discharge layers outside 1..KUB");
            for (int k = kmin; k <= kmax; ++k) {
                mohid::DischTerm t;
                t.k = k; t.kmin = kmin; t.kmax = kmax;
                t.flags = (uniform ? 1 : 0) | (ByPass[dis] ? 2 : 0);
                t.flow = DischFlow[n]; t.conc = DischConc[n]; t.concMF = DischConcMF[n];
                terms.push_back({i + sj * j, t, n});
            }
        }
    }
    // by column, then layer, keeping the reference's order among equal cells
    std::stable_sort(terms.begin(), terms.end(), [](const Term& x, const Term& y) {
        return x.col != y.col ? x.col < y.col : x.t.k < y.t.k;
    });
    std::vector<int> start(in->n2 + 1, 0);
    for (const auto& t : terms) ++start[(size_t)t.col + 1];
    for (size_t c = 0; c < in->n2; ++c) start[c + 1] += start[c];
    std::vector<mohid::DischTerm> tv(terms.size());
    for (size_t q = 0; q < terms.size(); ++q) tv[q] = terms[q].t;
    // host copies for the batched form (its own layout, a concentration per tracer)
    in->hTermCol.resize(terms.size());
    in->hTermCell.resize(terms.size());
    for (size_t q = 0; q < terms.size(); ++q) { in->hTermCol[q] = terms[q].col; in->hTermCell[q] = terms[q].cell; }
    in->hTerms = tv;
    in->nDischCells = n;
    CK(cudaSetDevice(in->device));
    CK(cudaStreamSynchronize(in->stream));              // no step still reads the old lists
    if (!in->dStart.p) {
        cudaError_t e = in->dStart.alloc(in->n2 + 1);
        if (e != cudaSuccess) return fail(MOHID_AD_ERR_ALLOC, stat, cuda_msg("cudaMalloc", e));
    }
    in->dTerms.release();
    if (!tv.empty()) {
        cudaError_t e = in->dTerms.alloc(tv.size());
        if (e != cudaSuccess) { in->hasDisch = false; return fail(MOHID_AD_ERR_ALLOC, stat, cuda_msg("cudaMalloc", e)); }
        CK(cudaMemcpy(in->dTerms.p, tv.data(), sizeof(mohid::DischTerm) * tv.size(), cudaMemcpyHostToDevice));
    }
    CK(cudaMemcpy(in->dStart.p, start.data(), sizeof(int) * start.size(), cudaMemcpyHostToDevice));
    in->hasDisch = !tv.empty();
    ++in->dischVersion;
    return ok(stat);
}

int mohid_ad_unset_discharges(const int* id, int* stat)
{
    Instance* in = lookup(id);
    if (!in) return fail(MOHID_AD_ERR_ID, stat, "unknown instance id");
    CK(cudaSetDevice(in->device));
    CK(cudaStreamSynchronize(in->stream));
    in->hasDisch = false;
    in->hTerms.clear(); in->hTermCol.clear(); in->hTermCell.clear();
    ++in->dischVersion;
    return ok(stat);
}

int mohid_ad_set_noflux(const int* id, const int* NoFluxU, const int* NoFluxV, const int* NoFluxW, int* stat)
{
    Instance* in = lookup(id);
    if (!in) return fail(MOHID_AD_ERR_ID, stat, "unknown instance id");
    if (!NoFluxU && !NoFluxV && !NoFluxW) {
        in->hasNoFlux = false;
        ++in->nofluxVersion;
        return ok(stat);
    }
    if (!NoFluxU || !NoFluxV || !NoFluxW) return fail(MOHID_AD_ERR_NULLPTR, stat, "give all three masks or none");
    CK(cudaSetDevice(in->device));
    DevBuf<int>* d[3] = {&in->NFU, &in->NFV, &in->NFW};
    const int* src[3] = {NoFluxU, NoFluxV, NoFluxW};
    for (int q = 0; q < 3; ++q) {
        if (!d[q]->p) {
            cudaError_t e = d[q]->alloc(in->n3);
            if (e != cudaSuccess) return fail(MOHID_AD_ERR_ALLOC, stat, cuda_msg("cudaMalloc", e));
        }
        CK(cudaMemcpyAsync(d[q]->p, src[q], sizeof(int) * in->n3, cudaMemcpyHostToDevice, in->stream));
    }
    CK(cudaStreamSynchronize(in->stream));
    in->hasNoFlux = true;
    ++in->nofluxVersion;
    return ok(stat);
}

// The PropOld argument of AdvectionDiffusion (AD:1139, AD:1253-1260), kept by
// pointer: steps with Orlanski boundaries write into it the field as
// OpenBoundaryCondition saw it (AD:5428-5429)
int mohid_ad_set_prop_old(const int* id, double* PropOld, const int* on_device, int* stat)
{
    Instance* in = lookup(id);
    if (!in) return fail(MOHID_AD_ERR_ID, stat, "unknown instance id");
    if (PropOld && !on_device) return fail(MOHID_AD_ERR_NULLPTR, stat, "on_device is NULL");
    in->propOld = PropOld;
    in->propOldDev = PropOld && *on_device != 0;
    return ok(stat);
}

// GetAdvFlux / GetDifFlux (AD:697-860): copies of the face fluxes of the
// last step, which must have been made with CellFluxes
static int get_fluxes(const int* id, int first, double* X, double* Y, double* Z, const int* on_device, int* stat)
{
    Instance* in = lookup(id);
    if (!in) return fail(MOHID_AD_ERR_ID, stat, "unknown instance id");
    if (!on_device) return fail(MOHID_AD_ERR_NULLPTR, stat, "NULL argument");
    if (!in->fluxLast || !in->flux.p)
        return fail(MOHID_AD_ERR_OPTION, stat, "the last step was not made with CellFluxes");
    CK(cudaSetDevice(in->device));
    const cudaMemcpyKind kind = *on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    double* dst[3] = {X, Y, Z};
    for (int q = 0; q < 3; ++q)
        if (dst[q])
            CK(cudaMemcpyAsync(dst[q], in->flux.p + (size_t)(first + q) * in->n3, sizeof(double) * in->n3, kind,
                               in->stream));
    CK(cudaStreamSynchronize(in->stream));
    return ok(stat);
}

int mohid_ad_get_adv_flux(const int* id, double* AdvFluxX, double* AdvFluxY, double* AdvFluxZ,
                          const int* on_device, int* stat)
{
    return get_fluxes(id, 0, AdvFluxX, AdvFluxY, AdvFluxZ, on_device, stat);
}

int mohid_ad_get_dif_flux(const int* id, double* DifFluxX, double* DifFluxY, double* DifFluxZ,
                          const int* on_device, int* stat)
{
    return get_fluxes(id, 3, DifFluxX, DifFluxY, DifFluxZ, on_device, stat);
}

int mohid_ad_debug_fail_alloc(const int* after, int* stat)
{
    if (!after) return fail(MOHID_AD_ERR_NULLPTR, stat, "NULL argument");
    if (*after < 0) return fail(MOHID_AD_ERR_BOUNDS, stat, "after must be >= 0");
    g_fail_alloc = *after;
    return ok(stat);
}

int mohid_ad_kill(int* id, int* stat)
{
    TraceRange trace_("mohid_ad_kill");
    Instance* in = nullptr;
    if (id) {
        std::lock_guard<std::mutex> lk(g_mu);
        auto it = g_inst.find(*id);
        if (it != g_inst.end()) { in = it->second; g_inst.erase(it); }
    }
    if (!in) return fail(MOHID_AD_ERR_ID, stat, "unknown instance id");
    cudaSetDevice(in->device);
    cudaStreamSynchronize(in->stream);
    in->release();
    delete in;
    *id = 0;
    return ok(stat);
}

int mohid_thomasz_f64(const int* ILB, const int* IUB, const int* JLB, const int* JUB,
                      const int* KLB, const int* KUB, const T_Size3D* size, const double* D,
                      const double* E, const double* F, const double* TI, double* RES,
                      const int* WaterPoints, int* stat)
{
    if (!ILB || !IUB || !JLB || !JUB || !KLB || !KUB || !size || !D || !E || !F || !TI || !RES || !WaterPoints)
        return fail(MOHID_AD_ERR_NULLPTR, stat, "mohid_thomasz_f64: NULL argument");
    if (*ILB != 1 || *JLB != 1 || *KLB != 1 || *IUB < 1 || *JUB < 1 || *KUB < 1 ||
        size->ILB != 0 || size->JLB != 0 || size->KLB != 0 || size->IUB != *IUB + 1 ||
        size->JUB != *JUB + 1 || size->KUB != *KUB + 1)
        return fail(MOHID_AD_ERR_BOUNDS, stat, "mohid_thomasz_f64: bounds must be WorkSize 1..N inside Size 0..N+1");
    if (*KUB > 200) return fail(MOHID_AD_ERR_UNSUPPORTED, stat, "KUB > 200 layers not supported");
    const int ni = *IUB, nj = *JUB, nk = *KUB;
    const size_t n3 = (size_t)(ni + 2) * (nj + 2) * (nk + 2);
    const size_t bd = n3 * sizeof(double);
    double *dD = nullptr, *dE = nullptr, *dF = nullptr, *dT = nullptr, *dR = nullptr;
    int* dW = nullptr;
    unsigned int* dS = nullptr;
    unsigned int hS = 0;
    cudaStream_t s = nullptr;
    int code = MOHID_AD_SUCCESS;
    std::string why;
    auto run = [&]() -> cudaError_t {
        cudaError_t e;
        if ((e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess) return e;
        double** bufs[] = {&dD, &dE, &dF, &dT, &dR};
        for (auto* b : bufs) if ((e = cudaMalloc((void**)b, bd)) != cudaSuccess) return e;
        if ((e = cudaMalloc((void**)&dW, n3 * sizeof(int))) != cudaSuccess) return e;
        if ((e = cudaMalloc((void**)&dS, sizeof(unsigned int))) != cudaSuccess) return e;
        const double* src[] = {D, E, F, TI, RES};
        double* dst[] = {dD, dE, dF, dT, dR};
        for (int q = 0; q < 5; ++q)
            if ((e = cudaMemcpyAsync(dst[q], src[q], bd, cudaMemcpyHostToDevice, s)) != cudaSuccess) return e;
        if ((e = cudaMemcpyAsync(dW, WaterPoints, n3 * sizeof(int), cudaMemcpyHostToDevice, s)) != cudaSuccess) return e;
        if ((e = cudaMemsetAsync(dS, 0, sizeof(unsigned int), s)) != cudaSuccess) return e;
        if ((e = mohid::launch_thomasz_f64(ni, nj, nk, dD, dE, dF, dT, dR, dW, dS, s)) != cudaSuccess) return e;
        if ((e = cudaMemcpyAsync(RES, dR, bd, cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
        if ((e = cudaMemcpyAsync(&hS, dS, sizeof(unsigned int), cudaMemcpyDeviceToHost, s)) != cudaSuccess) return e;
        return cudaStreamSynchronize(s);
    };
    cudaError_t e = run();
    double* bufs[] = {dD, dE, dF, dT, dR};
    for (double* b : bufs) if (b) cudaFree(b);
    if (dW) cudaFree(dW);
    if (dS) cudaFree(dS);
    if (s) cudaStreamDestroy(s);
    if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? MOHID_AD_ERR_ALLOC : MOHID_AD_ERR_CUDA, stat, cuda_msg("mohid_thomasz_f64", e));
    code = status_to_code(hS, why);
    if (code) return fail(code, stat, why);
    return ok(stat);
}

}  // extern "C"
