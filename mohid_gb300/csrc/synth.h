/*
 * synth.h -- seeded synthetic inputs for the advection-diffusion step
 * (benchmarks, tests and examples; not on the transport path).
 *
 * The generators restate the reference's geometry, mask and continuity rules
 * so that every field set is one MOHID itself could hand to AdvectionDiffusion.
 * Arrays are Fortran-ordered over the Size box (0:ni+1, 0:nj+1[, 0:nk+1]).
 */
#ifndef MOHID_SYNTH_H
#define MOHID_SYNTH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mohid_synth_params {
    int ni, nj, nk;
    double dx, dy;
    int zlevel;            /* 0 = uniform sigma layers, 1 = z-level (KFloor varies) */
    double hmin, hmax;     /* bathymetry range [m] */
    int bathy_kind;        /* 0 = ramp + Gaussian bump, 1 = smooth random, 2 = fractal */
    double land_frac;      /* target fraction of land columns */
    int land_kind;         /* 0 = western coastline block, 1 = smooth threshold, 2 = fractal threshold */
    double umax;           /* peak horizontal speed [m/s] */
    double visc_h;         /* Visc_H [m2/s] */
    double kz_median, kz_logsigma;  /* lognormal Diff_V */
    int open_sides;        /* bitmask: 1 west (j=1), 2 east (j=nj), 4 south (i=1), 8 north (i=ni) */
    double vol_var;        /* relative amplitude of VolumeZ - VolumeZOld (0 = fixed volumes) */
    double dt;             /* used for continuity with moving volumes */
    uint64_t seed;
} mohid_synth_params;

/* Writable views of the arrays the generator fills (Size box, Fortran order). */
typedef struct mohid_synth_out {
    double *DUX, *DVY, *DZX, *DZY;
    int *KFloorZ, *BoundaryPoints2D, *WaterPoints2D;
    double *Wflux_X, *Wflux_Y, *Wflux_Z, *VolumeZOld, *VolumeZ, *Visc_H, *Diff_V;
    double *AreaU, *AreaV, *DZZ, *DWZ;
    int *OpenPoints3D, *LandPoints3D, *WaterPoints3D;
    int *ComputeFacesU3D, *ComputeFacesV3D, *ComputeFacesW3D;
    double *depth;         /* 2-D bathymetry H(i,j) [m], 0 on land */
} mohid_synth_out;

/* Fill every array of *o.  Returns 0 or a negative error. */
int mohid_synth_generate(const mohid_synth_params* gp, mohid_synth_out* o);

/* Tracer initial fields (Size box, double).
 * kind 0: 3-D Gaussian, amplitude `a`, sigma `b` cells, seeded centre
 * kind 1: temperature-like a..b with a vertical gradient
 * kind 2: salinity-like a..b smooth horizontal field
 * kind 3: lognormal positive, median a, log-sigma b (smooth in space)
 * kind 4: constant a
 * Land and halo cells get 0. */
int mohid_synth_tracer(const mohid_synth_params* gp, const mohid_synth_out* o, int kind,
                    double a, double b, uint64_t seed, double* P);

/* Reference (exterior) concentration for open boundaries: a constant `c0`
 * plus a smooth seeded perturbation of relative amplitude `rel`. */
int mohid_synth_reference(const mohid_synth_params* gp, const mohid_synth_out* o, double c0,
                       double rel, uint64_t seed, double* R);

#ifdef __cplusplus
}
#endif
#endif
