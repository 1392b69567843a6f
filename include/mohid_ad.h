/*
 * mohid_ad.h -- C-ABI of the GB300 tracer advection-diffusion step.
 *
 * This is the drop-in boundary for MOHID Water's per-property transport call
 *   ModuleWaterProperties::Advection_Diffusion_Processes
 *     -> ModuleAdvectionDiffusion::AdvectionDiffusion
 *        (Software/MOHIDWater/ModuleWaterProperties.F90:14776-14824,
 *         Software/MOHIDBase2/ModuleAdvectionDiffusion.F90:1108-1509)
 * and for the legacy CUDA Thomas binding it supersedes
 *   SolveThomas_C / InitializeThomas_C / KillThomas_C
 *        (Software/CudaThomas/Thomas.h:11-27, Software/MOHIDBase1/ModuleCuda.F90:49-121).
 *
 * Conventions (Fortran ISO_C_BINDING friendly):
 *  - every scalar argument is passed by pointer (Fortran default by-reference);
 *  - every array is the base pointer of a Fortran column-major array over the
 *    `Size` box (ILB:IUB, JLB:JUB[, KLB:KUB]) with i fastest, exactly as MOHID
 *    allocates it (Size = WorkSize +/- 1 halo cell on every side,
 *    Software/MOHIDBase2/ModuleGeometry.F90:812-816);
 *  - REAL arrays are double precision: the reference Linux build promotes the
 *    default REAL to 8 bytes (-fdefault-real-8 / -real_size 64,
 *    Solutions/mohid-in-linux/compile_mohid.sh:185,209);
 *  - Fortran LOGICALs are passed as int (0 = .false., nonzero = .true.);
 *  - every entry point returns its status and also stores it in *stat
 *    (MOHID's STAT convention, SUCCESS_ = 0, Software/MOHIDBase1/ModuleGlobalData.F90:181).
 *    No entry point ever aborts the host process (the legacy CuExe called exit(1),
 *    Software/CudaWrapper/CuWrapper.cpp:11-19).
 *
 * Calls on one instance id must be serialised by the caller (MOHID calls the
 * transport inside its property loop, outside OpenMP regions); different ids may
 * be driven from different host threads -- each id owns its own CUDA stream.
 */
#ifndef MOHID_AD_H
#define MOHID_AD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define MOHID_AD_SUCCESS          0   /* SUCCESS_ (ModuleGlobalData.F90:181)                    */
#define MOHID_AD_ERR_BOUNDS       1   /* inconsistent Size/WorkSize bounds or array extents      */
#define MOHID_AD_ERR_ID           2   /* unknown / dead instance id (reference: ready_ /= IDLE)  */
#define MOHID_AD_ERR_OPTION       3   /* option combination the reference rejects with `stop`   */
#define MOHID_AD_ERR_UNSUPPORTED  4   /* option of the reference this library does not implement */
#define MOHID_AD_ERR_CUDA         5   /* CUDA runtime error (message via mohid_ad_last_error)    */
#define MOHID_AD_ERR_ZERO_PIVOT   6   /* THOMASZ pivot |E + D*W| == 0 in some water column       */
#define MOHID_AD_ERR_NONFINITE    7   /* a solved concentration is Inf/NaN                       */
#define MOHID_AD_ERR_ALLOC        8   /* device or pinned-host allocation failed                 */
#define MOHID_AD_ERR_NULLPTR      9   /* a required array pointer is NULL                        */
#define MOHID_AD_ERR_TIMEOUT     10   /* a bounded device-side wait gave up                      */

/* ---- option enums (values identical to the reference) ------------------ */
/* ModuleGlobalData.F90:1810-1811 */
#define MOHID_UPWIND_ORDER1   1
#define MOHID_UPWIND_ORDER2   2
#define MOHID_UPWIND_ORDER3   3
#define MOHID_P2_TVD          4
#define MOHID_CENTRAL_DIF     5
#define MOHID_LEAP_FROG       6
#define MOHID_TVD_MINMOD      1
#define MOHID_TVD_VANLEER     2
#define MOHID_TVD_MUSCL       3
#define MOHID_TVD_SUPERBEE    4
#define MOHID_TVD_PDM         5
/* ModuleAdvectionDiffusion.F90:152-158 */
#define MOHID_BC_MASS_CONSERVATION   1
#define MOHID_BC_IMPOSED_VALUE       2
#define MOHID_BC_NULL_GRADIENT       4
#define MOHID_BC_SUBMODEL            5
#define MOHID_BC_ORLANSKI            6
#define MOHID_BC_MASS_CONSERV_NULLGRAD 7
#define MOHID_BC_CYCLIC              8
/* ModuleGlobalData.F90:143 */
#define MOHID_NULL_REAL (-9.9e15)
/* face thickness options of ModuleGeometry (ModuleGeometry.F90:231-232) */
#define MOHID_FACES_AVERAGE_THICKNESS 2
#define MOHID_FACES_MIN_THICKNESS     3

/* T_Size3D, ModuleGlobalData.F90:2042-2052 (bind(c) under _USE_CUDA). */
typedef struct T_Size3D {
    int ILB, IUB, JLB, JUB, KLB, KUB;
} T_Size3D;

/*
 * Scalar arguments of AdvectionDiffusion (ModuleAdvectionDiffusion.F90:1108-1198),
 * same names and meaning.  `real` arguments are double (default REAL is 8 bytes
 * in the reference build).  Construction-time options of StartAdvectionDiffusion
 * (Vertical1D, XZFlow, Docycle_method; ModuleAdvectionDiffusion.F90:400-480) are
 * carried here too, so that one struct describes a call completely.
 */
typedef struct mohid_ad_params {
    double schmidt_H;             /* Schmidt number, horizontal                     */
    double SchmidtCoef_V;         /* Kz = SchmidtCoef_V * Diff_V + SchmidtBackground_V */
    double SchmidtBackground_V;
    int    AdvMethodH, TVDLimitationH;
    int    AdvMethodV, TVDLimitationV;
    int    Upwind2H, Upwind2V;    /* LOGICAL                                          */
    double VolumeRelMax;
    double DTProp;                /* property time step [s]                           */
    double ImpExp_AdvV;           /* 1 = implicit (default), 0 = explicit             */
    double ImpExp_DifV;           /* 1 = implicit, 0 = explicit, in between = theta   */
    double ImpExp_AdvXX;          /* 0 explicit, 1 implicit (plain form only)         */
    double ImpExp_AdvYY;          /* 0 explicit, 1 implicit (plain form only)         */
    double ImpExp_DifH;           /* must be 0: the reference requires explicit H-diff */
    int    NullDif;               /* LOGICAL                                          */
    int    BoundaryCondition;     /* MOHID_BC_*; 4 and 8 also act without a reference */
    double DecayTime;             /* [s]                                              */
    int    AdvectionNudging;      /* LOGICAL: nudging near open boundaries (plain form) */
    int    AdvectionNudgingCells;
    int    CellFluxes;            /* LOGICAL: record the face fluxes                  */
    int    NoAdvFlux, NoDifFlux;  /* LOGICAL: use the NoFlux masks                    */
    int    Optimize, FirstProperty; /* LOGICAL; accepted, results follow the general path */
    int    Vertical1D, XZFlow;    /* LOGICAL, StartAdvectionDiffusion options          */
    int    Docycle_method;        /* 1 (default) or 2, ModuleModel.F90:641-646        */
} mohid_ad_params;

/* Fill *p with the reference's defaults (ModuleWaterProperties.F90:9305-9680):
 * UpwindOrder1 H and V, SuperBee limiters, Upwind2H/V false, VolumeRelMax 1.5,
 * Schmidt numbers 1, background 1e-8, implicit V advection and diffusion,
 * explicit H, MassConservation, DecayTime 0, Docycle_method 1. */
void mohid_ad_default_params(mohid_ad_params* p);

/* Text of the last error on this host thread (never NULL). */
const char* mohid_ad_last_error(void);

/* Library version string, e.g. "mohid-gb300 0.1 sm_103a". */
const char* mohid_ad_version(void);

/* ======================================================================== */
/* Plain FP64 drop-in (one property per call, Fortran layout, in place)      */
/* ======================================================================== */

/*
 * Construct an instance: StartAdvectionDiffusion (ModuleAdvectionDiffusion.F90:400)
 * plus the grid getters AdvectionDiffusion performs each call
 * (GetHorizontalGrid DUX/DVY/DZX/DZY, GetBoundaries, GetGeometryKFloor;
 * ModuleAdvectionDiffusion.F90:1353-1401).  The static 2-D metrics are
 * uploaded once.  `size` is the allocation box, `worksize` the computed box;
 * size must equal worksize +/- 1 in i, j and k.
 *   DUX, DVY, DZX, DZY : double (ILB:IUB, JLB:JUB)
 *   KFloorZ, BoundaryPoints2D : int (ILB:IUB, JLB:JUB)
 * On success *id > 0.
 */
int mohid_ad_init(int* id, const T_Size3D* size, const T_Size3D* worksize,
                  const double* DUX, const double* DVY,
                  const double* DZX, const double* DZY,
                  const int* KFloorZ, const int* BoundaryPoints2D, int* stat);

/*
 * Upload the fields shared by every property of one time step (the arguments
 * of AdvectionDiffusion that do not depend on the property).  All 3-D arrays
 * are over the Size box.  `SmallDepths` (int, 2-D) may be NULL.
 * Equivalent to the pointer-binding part of the reference call; lets a caller that
 * transports N properties per step send the hydrodynamics once instead of N times.
 * After the first call any of the eleven FP64 arrays may be NULL: the instance
 * keeps its copy (unchanged since the last call, or made on the device by
 * mohid_ad_geometry_dev / mohid_ad_vertical_flux).  The six 3-D masks are given
 * all together (then checked, and SmallDepths replaced) or all NULL (kept,
 * SmallDepths ignored); a call that keeps the masks does not wait for the
 * device beyond consuming the host buffers.
 */
int mohid_ad_set_hydro(const int* id,
                       const double* Wflux_X, const double* Wflux_Y, const double* Wflux_Z,
                       const double* VolumeZOld, const double* VolumeZ,
                       const double* Visc_H, const double* Diff_V,
                       const double* AreaU, const double* AreaV,
                       const double* DZZ, const double* DWZ,
                       const int* OpenPoints3D, const int* LandPoints3D,
                       const int* WaterPoints3D,
                       const int* ComputeFacesU3D, const int* ComputeFacesV3D,
                       const int* ComputeFacesW3D,
                       const int* SmallDepths, int* stat);

/*
 * Transport one property over one step with the hydrodynamics of the last
 * mohid_ad_set_hydro call: PROP (double, Size box) is read and overwritten in
 * place, as AdvectionDiffusion does (THOMASZ_NewType2's RES aliases PROP,
 * ModuleFunctions.F90:4026-4123).  ReferenceProp may be NULL (closed
 * boundaries); when given, `p->BoundaryCondition` selects the open-boundary
 * treatment (ModuleAdvectionDiffusion.F90:5369-5742): MassConservation,
 * ImposedValue, SubModel, Orlanski, NullGradient, MassConservNullGrad or
 * Cyclic.  Orlanski radiates the field outwards (OrlanskiCelerity2D,
 * ModuleFunctions.F90:4129-4490): the exterior point of each open boundary
 * cell (a halo cell, or for the corner i = IUB, j = JLB the interior point
 * IUB-1) takes the radiated value, which the boundary cell's inflow carries
 * in; a boundary point off the work box's edges returns MOHID_AD_ERR_OPTION
 * (the reference stops), a grid under 3 cells wide whose radiation would read
 * outside the layer plane MOHID_AD_ERR_BOUNDS.  As in the reference,
 * NullGradient sets the boundary columns to their neighbours' mean after the
 * solve whether or not ReferenceProp is given (AD:1874-1987), and Cyclic
 * (AD:2121-2224) needs ReferenceProp (MOHID_AD_ERR_OPTION without it).
 */
int mohid_ad_step_prop_f64(const int* id, double* PROP, const double* ReferenceProp,
                           const mohid_ad_params* p, int* stat);

/*
 * SetDischarges / UnSetDischarges (ModuleAdvectionDiffusion.F90:978-1075):
 * point sources applied by the following steps right after VolumeVariation
 * (AD:4025-4128).  Per discharge (*DischNumber of them): DischnCells,
 * IgnoreDisch, ByPass (LOGICAL as int) and DischVert (5 = DischUniform_:
 * the flow is spread over layers Kmin..Kmax by thickness, -9999999 =
 * FillValueInt reads as KFloorZ / KUB; any other value: layer DischK).  Per
 * cell of the discharges not ignored, in order: DischI, DischJ, DischK,
 * DischKmin, DischKmax (work-box indices), DischFlow, DischConc, DischConcMF.
 * The arguments are copied.  Cells outside the work box or layers outside
 * 1..KUB return MOHID_AD_ERR_BOUNDS.  DischConc is per property, so call it
 * before each property's step as WP does.
 */
int mohid_ad_set_discharges(const int* id, const int* DischNumber, const int* DischnCells, const int* IgnoreDisch,
                            const int* ByPass, const int* DischVert, const int* DischI, const int* DischJ,
                            const int* DischK, const int* DischKmin, const int* DischKmax, const double* DischFlow,
                            const double* DischConc, const double* DischConcMF, int* stat);
int mohid_ad_unset_discharges(const int* id, int* stat);

/*
 * The NoFluxU / NoFluxV / NoFluxW masks of AdvectionDiffusion's optional
 * arguments (Size-box int arrays, host).  Steps with p->NoAdvFlux zero the
 * advection coefficients of masked faces, and steps with p->NoDifFlux their
 * horizontal diffusivities and vertical diffusion conductances (AD:2496,
 * 2527, 2741, 3004, 4434, 4804).  They need all three masks
 * (MOHID_AD_ERR_NULLPTR otherwise).  All three NULL clears them.
 */
int mohid_ad_set_noflux(const int* id, const int* NoFluxU, const int* NoFluxV, const int* NoFluxW, int* stat);

/*
 * The PropOld argument of AdvectionDiffusion (ModuleAdvectionDiffusion.F90:1139,
 * 1253-1260).  Steps with Orlanski boundaries (BoundaryCondition 6 and a
 * ReferenceProp) write into it the field as OpenBoundaryCondition saw it,
 * PROPOld(:,:,:) = PROP(:,:,:) (AD:5428-5429): the step's input, or with
 * implicit horizontal advection the line solution.  OrlanskiCelerity2D reads
 * it as the previous time level.  Host (*on_device == 0) or device array over
 * the Size box, kept by pointer: it must stay valid while steps run.  NULL
 * detaches it; other boundary conditions leave it untouched.
 */
int mohid_ad_set_prop_old(const int* id, double* PropOld, const int* on_device, int* stat);

/*
 * GetAdvFlux / GetDifFlux (ModuleAdvectionDiffusion.F90:697-860): the face
 * fluxes of the instance's last step, which must have been made with
 * p->CellFluxes (MOHID_AD_ERR_OPTION otherwise).  Size-box arrays: the flux
 * through the west (X: between j-1 and j), south (Y: between i-1 and i) and
 * bottom (Z: between k-1 and k) face of each cell, positive towards the cell;
 * zero away from compute faces.  Explicit parts use the field as the
 * explicit term saw it, implicit parts the new field (AD:1882-1916).  Any of
 * the three pointers may be NULL; host (*on_device == 0) or device arrays.
 */
int mohid_ad_get_adv_flux(const int* id, double* AdvFluxX, double* AdvFluxY, double* AdvFluxZ,
                          const int* on_device, int* stat);
int mohid_ad_get_dif_flux(const int* id, double* DifFluxX, double* DifFluxY, double* DifFluxZ,
                          const int* on_device, int* stat);

/*
 * All-in-one drop-in with the argument surface of AdvectionDiffusion:
 * mohid_ad_set_hydro + mohid_ad_step_prop_f64.
 */
int mohid_ad_step_f64(const int* id, double* PROP, const mohid_ad_params* p,
                      const double* Wflux_X, const double* Wflux_Y, const double* Wflux_Z,
                      const double* VolumeZOld, const double* VolumeZ,
                      const double* Visc_H, const double* Diff_V,
                      const double* AreaU, const double* AreaV,
                      const double* DZZ, const double* DWZ,
                      const int* OpenPoints3D, const int* LandPoints3D,
                      const int* WaterPoints3D,
                      const int* ComputeFacesU3D, const int* ComputeFacesV3D,
                      const int* ComputeFacesW3D,
                      const int* SmallDepths,
                      const double* ReferenceProp, int* stat);

/*
 * Device-resident variant of mohid_ad_step_prop_f64: PROP_in and PROP_out are
 * device pointers (Size box, double), distinct; the call is asynchronous on the
 * instance's stream (query it with mohid_ad_stream).  Every cell of PROP_out is
 * written (cells the reference leaves untouched are copied from PROP_in).
 * ReferenceProp, if not NULL, is a device pointer.  Device-side failures
 * (zero pivot, non-finite result) are latched and reported by
 * mohid_ad_sync.
 */
int mohid_ad_step_prop_f64_dev(const int* id, const double* PROP_in, double* PROP_out,
                               const double* ReferenceProp,
                               const mohid_ad_params* p, int* stat);

/* Upload hydrodynamics that already live on the device (same layout and
 * NULL rules as mohid_ad_set_hydro, device pointers; copied device-to-device,
 * asynchronous when the masks are kept). */
int mohid_ad_set_hydro_dev(const int* id,
                           const double* Wflux_X, const double* Wflux_Y, const double* Wflux_Z,
                           const double* VolumeZOld, const double* VolumeZ,
                           const double* Visc_H, const double* Diff_V,
                           const double* AreaU, const double* AreaV,
                           const double* DZZ, const double* DWZ,
                           const int* OpenPoints3D, const int* LandPoints3D,
                           const int* WaterPoints3D,
                           const int* ComputeFacesU3D, const int* ComputeFacesV3D,
                           const int* ComputeFacesW3D,
                           const int* SmallDepths, int* stat);

/* The eleven FP64 fields as borrowed device arrays, as AdvectionDiffusion
 * binds its array arguments by pointer (ModuleAdvectionDiffusion.F90:1271-1292):
 * the instance reads them in place, with no copy, until the next
 * mohid_ad_set_hydro* or mohid_ad_bind_hydro_dev call gives that field
 * again, and the device producers (mohid_ad_geometry_dev,
 * mohid_ad_vertical_flux) write their results into them.  They must stay
 * valid and must not change while a step that reads them runs; after
 * changing their contents call this again (with the same pointers), which
 * marks the hydrodynamic state as new.  NULL and mask rules as
 * mohid_ad_set_hydro_dev; the masks are copied. */
int mohid_ad_bind_hydro_dev(const int* id,
                            const double* Wflux_X, const double* Wflux_Y, const double* Wflux_Z,
                            const double* VolumeZOld, const double* VolumeZ,
                            const double* Visc_H, const double* Diff_V,
                            const double* AreaU, const double* AreaV,
                            const double* DZZ, const double* DWZ,
                            const int* OpenPoints3D, const int* LandPoints3D,
                            const int* WaterPoints3D,
                            const int* ComputeFacesU3D, const int* ComputeFacesV3D,
                            const int* ComputeFacesW3D,
                            const int* SmallDepths, int* stat);

/* Copy the instance's current FP64 hydrodynamic fields (those of the last
 * mohid_ad_set_hydro*, as changed since by the device producers) to the
 * caller's Size-box arrays; any pointer may be NULL (not copied).  Host
 * pointers when *on_device == 0, device pointers otherwise.  Synchronous. */
int mohid_ad_get_hydro(const int* id, double* Wflux_X, double* Wflux_Y, double* Wflux_Z,
                       double* VolumeZOld, double* VolumeZ, double* Visc_H, double* Diff_V,
                       double* AreaU, double* AreaV, double* DZZ, double* DWZ,
                       const int* on_device, int* stat);

/* Wait for the instance's stream and report latched device errors. */
int mohid_ad_sync(const int* id, int* stat);

/* The instance's cudaStream_t, as an opaque pointer. */
void* mohid_ad_stream(const int* id);

/* KillAdvectionDiffusion (ModuleAdvectionDiffusion.F90:5849): free the instance. */
int mohid_ad_kill(int* id, int* stat);

/* ======================================================================== */
/* Batched FP32 form: many tracers of one property group per call            */
/* ======================================================================== */

/*
 * A batch transports `ntracers` properties that share the grid, the
 * hydrodynamics and the option set of plain instance `id` (one MOHID property
 * group: Advection_Diffusion_Processes calls AdvectionDiffusion once per
 * property with the same fluxes, volumes and masks, WP:14603-14824).  Tracers
 * stay on the device in FP32 ping-pong buffers; arithmetic is FP32 except the
 * volume difference V - Vold (FP64) and the mass budget (FP64, compensated).
 *   storage: 0 = FP32 transports and diffusivities,
 *            1 = FP16 transports with a per-field scale,
 *            2 = FP16 transports and diffusivities with per-field scales.
 * Supported options: AdvMethodH UpwindOrder1 or P2_TVD (any limiter),
 * explicit horizontal advection, implicit upwind vertical advection,
 * implicit vertical diffusion, Docycle_method 1; closed boundaries or the
 * open boundaries MassConservation, ImposedValue, NullGradient, SubModel,
 * MassConservNullGrad and Cyclic; discharges
 * (mohid_ad_batched_set_discharge_conc); the NoFlux masks on batches without
 * references; CellFluxes (mohid_ad_batched_get_adv_flux / _dif_flux).
 * Other options (Orlanski boundaries, AdvectionNudging, implicit horizontal
 * advection among them) return MOHID_AD_ERR_UNSUPPORTED (use the plain form).
 */
int mohid_ad_batched_create(int* bid, const int* id, const int* ntracers, const int* storage, int* stat);

/* Repack the plain instance's current hydrodynamics (mohid_ad_set_hydro[_dev])
 * into the batched layout.  mohid_ad_batched_step does this itself when the
 * hydrodynamics changed since the last pack. */
int mohid_ad_batched_pack_hydro(const int* bid, int* stat);

/* Load / read tracer t (0-based) from / to a Fortran-layout double array over
 * the Size box, on the host (*on_device == 0) or on the device. */
int mohid_ad_batched_set_tracer(const int* bid, const int* t, const double* PROP, const int* on_device, int* stat);
int mohid_ad_batched_get_tracer(const int* bid, const int* t, double* PROP, const int* on_device, int* stat);

/*
 * Discharge concentrations of tracer t (0-based): DischConc of SetDischarges
 * (ModuleAdvectionDiffusion.F90:978-1075), one value per discharge cell of the
 * plain instance's mohid_ad_set_discharges call and in its order; WP calls
 * SetDischarges per property with that property's concentrations
 * (WP:14763-14770).  The cells, flows, withdrawal factors (DischConcMF, which
 * the tracers share), vertical distribution and bypass flags are those of
 * mohid_ad_set_discharges.  With discharges set on the plain instance every
 * tracer needs its concentrations before a step (MOHID_AD_ERR_OPTION
 * otherwise); the tracers are then held as absolute values and the mass fixer
 * does not run (the discharges add and remove mass).  Ensembles reject
 * members with discharges.
 */
int mohid_ad_batched_set_discharge_conc(const int* bid, const int* t, const double* DischConc, int* stat);

/*
 * GetAdvFlux / GetDifFlux (ModuleAdvectionDiffusion.F90:697-860) of tracer t
 * (0-based) of the batch: the face fluxes of its last step, which the last
 * mohid_ad_batched_step call must have made with p->CellFluxes
 * (MOHID_AD_ERR_OPTION otherwise, and after the tracer or the hydrodynamics
 * were loaded again).  Same arrays and conventions as mohid_ad_get_adv_flux /
 * mohid_ad_get_dif_flux; FP32 arithmetic.  They are formed on request from
 * the field before and after that step, so steps with CellFluxes cost nothing
 * more.  Ensembles reject CellFluxes.
 */
int mohid_ad_batched_get_adv_flux(const int* bid, const int* t, double* AdvFluxX, double* AdvFluxY,
                                  double* AdvFluxZ, const int* on_device, int* stat);
int mohid_ad_batched_get_dif_flux(const int* bid, const int* t, double* DifFluxX, double* DifFluxY,
                                  double* DifFluxZ, const int* on_device, int* stat);

/* Exterior (reference) concentration of tracer t for open boundaries
 * (ReferenceProp of AdvectionDiffusion); once set for any tracer, every
 * tracer of the batch uses open boundaries and must have one.  Set it after
 * the tracer itself: a tracer is held as its anomaly from a per-tracer
 * constant (the mean over its water cells, chosen when it is loaded), and
 * its reference is stored relative to the same constant (the step subtracts
 * the mass fixer's correction to that constant).  Only the boundary columns
 * (BoundaryPoints2D == 1) read a reference, so only they are kept: (KUB + 2)
 * FP32 values per boundary column and tracer. */
int mohid_ad_batched_set_reference(const int* bid, const int* t, const double* ReferenceProp,
                                   const int* on_device, int* stat);

/* Advance every tracer *nsteps steps with options *p, asynchronously on the
 * plain instance's stream.  *use_graph != 0 captures the step loop in a CUDA
 * graph (re-used while nsteps, the options and the buffer parity match). */
int mohid_ad_batched_step(const int* bid, const mohid_ad_params* p, const int* nsteps, const int* use_graph,
                          int* stat);

/* Autotuner.  No counterpart in the reference.  Times each launch schedule of
 * the batch on the batch itself and keeps the fastest.  The schedules are one
 * CTA per tile, or a persistent grid over the tiles that hold water with the
 * deepest first (the column-length-aware schedule for z-level domains); tiles
 * of 32 columns by 8 or by 4 rows (a warp per row); with 4 or more tracers, 4
 * or 2 tracers per launch (with 8 or more also 8, with 10 or more also 10).
 * Each candidate runs a warm-up and two timed steps that leave the tracers
 * unchanged, in two rounds over all candidates; each keeps its faster time.
 * The first mohid_ad_batched_step of a batch runs it; call it again after a
 * change that may favour another schedule. */
int mohid_ad_batched_autotune(const int* bid, const mohid_ad_params* p, int* stat);

/* Set the schedule by hand (*sched 0 or 1, *split 10, 8, 4 or 2, *tile_rows 8
 * or 4; tile_rows NULL keeps the tile height) instead of the autotuner. */
int mohid_ad_batched_set_schedule(const int* bid, const int* sched, const int* split, const int* tile_rows,
                                  int* stat);

/* The schedule in use: kernel launches per step (the step kernels, and with
 * open boundaries the boundary flux and the mass fixer's finish), schedule (0
 * one CTA per tile, 1 tile list), largest tracer group per launch, and
 * launches made once per mohid_ad_batched_step call (the mass fixer's finish on
 * closed domains, which runs after the call's last step only), and the tile
 * height (rows of 32 columns).  Any output pointer may be NULL. */
int mohid_ad_batched_schedule(const int* bid, int* launches, int* sched, int* split, int* per_call,
                              int* tile_rows, int* stat);

/* Mass fixer (*on != 0, the default).  No counterpart in the reference, whose
 * FP64 arithmetic conserves mass to round-off; it restores that for the FP32
 * form.  After every step each tracer's mass (compensated sum of VolumeZ *
 * PROP over water cells, accumulated in the step kernel) is brought to its
 * target by adding one FP64 constant to every water cell, which leaves the
 * step's result otherwise unchanged.  The target is the FP64 mass of the
 * field as loaded plus, with MassConservation open boundaries, the mass the
 * steps moved through them since (FluxAtOpenBoundary: WFOB * DT times the
 * inflow concentration where WFOB < 0 and times the new value where
 * WFOB >= 0, summed in FP64 over the open boundary cells).  It runs where the
 * reference's budget closes exactly: a step that maps constants onto
 * themselves (continuity holds, XZFlow and Vertical1D off) and VolumeZ ==
 * VolumeZOld on every cell.  A new hydrodynamic state whose VolumeZ differs
 * from the last one ends it for the tracers loaded before that state (their
 * target no longer applies); tracers loaded afterwards keep it.  With open
 * boundaries, a step made without the fixer ends it for every tracer loaded
 * before.  Elsewhere the step runs without it. */
int mohid_ad_batched_set_mass_fix(const int* bid, const int* on, int* stat);

/* Mass that entered tracer t through open boundaries since it was loaded, as
 * the mass fixer's target followed it: mass = loaded mass + *flux while the
 * fixer runs (0 on closed domains), NaN once the fixer stopped for the tracer
 * (synchronous).  No counterpart in the reference. */
int mohid_ad_batched_boundary_flux(const int* bid, const int* t, double* flux, int* stat);

/* Global mass budget of tracer t: Neumaier-compensated FP64 sum of
 * VolumeZ * PROP over water cells (synchronous). */
int mohid_ad_batched_mass(const int* bid, const int* t, double* mass, int* stat);

/* Wait for the batch's stream and report latched device errors. */
int mohid_ad_batched_sync(const int* bid, int* stat);

int mohid_ad_batched_destroy(int* bid, int* stat);

/* ---- test hooks (no counterpart in the reference; failure detection is
 * tested by injecting on the host and by waits that run out, never by a GPU
 * fault) */

/* The *after-th device allocation from now fails with MOHID_AD_ERR_ALLOC
 * (0: off), to exercise the cleanup of every allocating entry point. */
int mohid_ad_debug_fail_alloc(const int* after, int* stat);

/* Runs the step kernels' bounded stage wait on a barrier that nothing
 * completes, for *polls polls: returns MOHID_AD_ERR_TIMEOUT, the status a
 * step reports when a stage never arrives. */
int mohid_ad_debug_wait_probe(const int* polls, int* stat);

/* ======================================================================== */
/* Ensemble: many independent batched domains in one launch                  */
/* ======================================================================== */

/*
 * No counterpart in the reference, which runs one domain per process (nested
 * and ensemble runs of MOHID Water are separate model instances).  An
 * ensemble steps *nmembers batches (bids[0..nmembers-1]) together: one
 * persistent grid walks the tiles of every member, largest layer count first.
 * Members must live on the same device and have the same tracer count (1, 2
 * or 4) and FP32 storage (storage 0); each keeps its own grid, hydrodynamics,
 * tracers, DT and options.  Members stay usable as batches (set_tracer,
 * get_tracer, mass); do not step a member on its own while it is in an
 * ensemble.  The ensemble runs on the stream of the first member's instance.
 */
int mohid_ad_ensemble_create(int* eid, const int* nmembers, const int* bids, int* stat);

/* Advance every member *nsteps steps, member m with options p[m] (same
 * AdvMethodH and TVDLimitationH for all members).  *use_graph != 0 captures
 * the step loop in a CUDA graph, as mohid_ad_batched_step does. */
int mohid_ad_ensemble_step(const int* eid, const mohid_ad_params* p, const int* nsteps, const int* use_graph,
                           int* stat);

/* Release the ensemble (the member batches are not destroyed). */
int mohid_ad_ensemble_destroy(int* eid, int* stat);

/* ======================================================================== */
/* Device producers of the step's geometry and vertical water flux           */
/* ======================================================================== */

/*
 * The geometry of a new water level on the instance's device arrays, as
 * ModuleGeometry computes it before the transport call
 * (Software/MOHIDBase2/ModuleGeometry.F90): StoreVolumeZOld (GEO:4335-4370)
 * when *store_old != 0, then ComputeDistances (GEO:3798-4103: DWZ = SZZ(k-1) -
 * SZZ(k) on water points, the face thicknesses DUZ / DVZ between water points,
 * minimum or DUX/DVY-weighted by *faces_option, DZZ = (DWZ(k+1) + DWZ(k)) / 2),
 * ComputeVolumes (GEO:4108-4163: VolumeZ = DWZ * DUX * DVY) and ComputeAreas
 * (GEO:4238-4288: AreaU = DUZ * DYY, AreaV = DVZ * DXX; without
 * impermeability).  SZZ: layer interface depths (Size box), DXX, DYY (2-D Size
 * box), all device pointers; WaterPoints3D is the one of the last
 * mohid_ad_set_hydro*, DUX / DVY those of mohid_ad_init.  Every value is the
 * reference's, bit for bit; arrays keep their values where the reference does
 * not write them.  Asynchronous on the instance's stream.
 */
int mohid_ad_geometry_dev(const int* id, const double* SZZ, const double* DXX, const double* DYY,
                          const int* faces_option, const int* store_old, int* stat);

/*
 * The vertical water flux of the instance from continuity, in place
 * (ModuleHydrodynamic.F90 WaterFlux_Z_VarGrid HD:43270-43308 when
 * *var_grid != 0, WaterFlux_Z_FixGrid HD:43315-43349 otherwise): on every
 * water point, Wflux_Z(k+1) = Wflux_Z(k) + West - East + South - North
 * [- (VolumeZ - VolumeZOld) / DT], from the instance's horizontal fluxes,
 * volumes and compute-face masks.  Wflux_Z at each column's floor is kept.
 * Asynchronous on the instance's stream.
 */
int mohid_ad_vertical_flux(const int* id, const double* DT, const int* var_grid, int* stat);

/* ======================================================================== */
/* Stand-alone THOMASZ (replaces SolveThomas_C with dim = 2 = Z)             */
/* ======================================================================== */

/*
 * Solve THOMASZ_NewType2 (ModuleFunctions.F90:4026-4123) for every column
 * (i,j) of the work box with WaterPoints(i,j,KUB) == 1, rows KLB..KUB+1,
 * exactly as the reference's CPU routine and the legacy CUDA path
 * (SolveThomas_C, Software/CudaThomas/Thomas.cu:23-51, 464-491) do.
 *   ILB..KUB  : WORK box bounds (the arguments the reference passes)
 *   size      : allocation box of D, E, F, TI, RES, WaterPoints
 *   D, E, F, TI : double (Size box), host pointers
 *   RES        : double (Size box), host pointer, written for solved columns
 * Columns not solved are left untouched.
 */
int mohid_thomasz_f64(const int* ILB, const int* IUB, const int* JLB, const int* JUB,
                      const int* KLB, const int* KUB, const T_Size3D* size,
                      const double* D, const double* E, const double* F,
                      const double* TI, double* RES, const int* WaterPoints, int* stat);

/* ======================================================================== */
/* Mass budget without allocation                                            */
/* ======================================================================== */

/*
 * No counterpart in the reference.  Global mass budget of one property:
 * Neumaier-compensated FP64 sum of VolumeZ * PROP over the water cells
 * (WaterPoints3D == 1) of the work box, written to *mass.  All pointers are
 * device pointers over the Size box (0:IUB, 0:JUB, 0:KUB of `size`); the call is
 * asynchronous on `stream` (a cudaStream_t, NULL for the default stream).
 *
 * For callers that cannot allocate device memory when they need the budget --
 * a model whose device memory belongs to another allocator (a caching
 * allocator that already holds the GPU, or a fixed budget reserved at start-up)
 * or one that must not synchronise the device inside its time step -- this
 * entry point allocates nothing: its scratch is a file-scope device array of
 * 2 x 8192 doubles (128 KiB).  A GPU holds it from the first call on that
 * device (which loads the library's CUDA module, lazily, and looks the array
 * up with cudaGetSymbolAddress) until the process exits.  That first call can
 * synchronise, or fail under memory pressure, as any module load can: make it
 * at start-up (a warm-up call), before any stream capture and outside the time
 * step.  The lookup is repeated only when the calling thread's CUDA context
 * changes (a reset primary context, another context on the device).
 * Limit: at most 8192 work-box rows (JUB - 1 <= 8192); larger grids return
 * MOHID_AD_ERR_BOUNDS.  Calls share the array, so calls that overlap on the
 * GPU (other streams or other host threads) race; every call overwrites the
 * part it reads, so nothing needs clearing between calls.
 */
int mohid_ad_mass_f64_noalloc(const T_Size3D* size, const double* PROP, const double* VolumeZ,
                              const int* WaterPoints3D, double* mass, void* stream, int* stat);

#ifdef __cplusplus
}
#endif

#endif /* MOHID_AD_H */
