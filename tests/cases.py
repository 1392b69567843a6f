"""Seeded small domains and option sets shared by the parity tests."""
import numpy as np

from mohid_gb300 import synth

# small grids: coastline block, z-level uneven columns, open boundaries with
# moving volumes, single layer (2-D), fully open, single column
SMALL = {
    "coast": dict(ni=7, nj=9, nk=5, land_frac=0.2, land_kind=0, seed=3),
    "zlevel": dict(ni=8, nj=6, nk=6, land_frac=0.25, land_kind=1, seed=4, zlevel=True,
                   hmin=2.0, hmax=60.0, bathy_kind=2),
    "open": dict(ni=9, nj=8, nk=4, land_frac=0.1, land_kind=1, seed=5, open_sides=3,
                 vol_var=0.01, bathy_kind=1),
    "layer1": dict(ni=6, nj=7, nk=1, land_frac=0.0, seed=6),
    "nsopen": dict(ni=10, nj=6, nk=3, land_frac=0.0, seed=7, open_sides=12, bathy_kind=1),
    "column": dict(ni=1, nj=1, nk=8, land_frac=0.0, seed=8),
}

# AdvectionDiffusion option sets (non-default values only)
OPTIONS = {
    "upwind1": dict(),
    "tvd_superbee": dict(AdvMethodH=4, TVDLimitationH=4, Upwind2H=1),
    "tvd_minmod": dict(AdvMethodH=4, TVDLimitationH=1, Upwind2H=1),
    "tvd_vanleer": dict(AdvMethodH=4, TVDLimitationH=2, Upwind2H=1),
    "tvd_muscl": dict(AdvMethodH=4, TVDLimitationH=3, Upwind2H=1),
    "tvd_pdm": dict(AdvMethodH=4, TVDLimitationH=5, Upwind2H=1),
    "upwind2": dict(AdvMethodH=2, Upwind2H=1),
    "upwind3": dict(AdvMethodH=3, Upwind2H=1),
    "central": dict(AdvMethodH=5),
    "leapfrog": dict(AdvMethodH=6),
    "tvd_vertical": dict(AdvMethodV=4, TVDLimitationV=4, Upwind2V=1),
    "explicit_v_tvd": dict(ImpExp_AdvV=0.0, AdvMethodV=4, TVDLimitationV=1, Upwind2V=1),
    "explicit_v_up3": dict(ImpExp_AdvV=0.0, AdvMethodV=3, Upwind2V=1),
    "theta_difv": dict(ImpExp_DifV=0.5),
    "explicit_difv": dict(ImpExp_DifV=0.0),
    "docycle2": dict(Docycle_method=2),
    "nulldif": dict(NullDif=1),
    "vertical1d": dict(Vertical1D=1),
    "xzflow": dict(XZFlow=1),
    "background": dict(SchmidtBackground_V=1e-3, schmidt_H=0.7, SchmidtCoef_V=2.0),
    "implicit_xx": dict(ImpExp_AdvXX=1.0),
    "implicit_yy_tvd": dict(ImpExp_AdvYY=1.0, AdvMethodH=4, TVDLimitationH=4, Upwind2H=1),
    "implicit_xx_central": dict(ImpExp_AdvXX=1.0, AdvMethodH=5),
}


def domain(name, dt=30.0):
    return synth.generate(synth.GenSpec(**SMALL[name], dt=dt))


def boundary_flux(d, P_old, P_new, ref, DT, decay_time=0.0, gross=False):
    """Mass moved through MassConservation open boundaries in one step
    (AdvectionDiffusion FluxAtOpenBoundary / OpenBoundaryCondition): at every
    open cell of a boundary column, WFOB = net face transport into the cell less
    (VolumeZ - VolumeZOld) / DT; the cell gains -WFOB * DT * Ext where WFOB < 0
    (Ext: the reference blended with the old value by the decay factor) and
    loses WFOB * DT * P_new where WFOB >= 0.  FP64, from the domain arrays.
    gross: also the sum of the cells' absolute gains and losses."""
    a = d.arrays
    nk, nj, ni = d.nk, d.nj, d.ni
    qx = a["Wflux_X"] * a["ComputeFacesU3D"]
    qy = a["Wflux_Y"] * a["ComputeFacesV3D"]
    qz = a["Wflux_Z"] * a["ComputeFacesW3D"]
    c = (slice(1, nk + 1), slice(1, nj + 1), slice(1, ni + 1))
    w = (qx[c] - qx[1:nk + 1, 2:nj + 2, 1:ni + 1] + qy[c] - qy[1:nk + 1, 1:nj + 1, 2:ni + 2] + qz[c] -
         qz[2:nk + 2, 1:nj + 1, 1:ni + 1] - (a["VolumeZ"][c] - a["VolumeZOld"][c]) / DT)
    kk = np.arange(1, nk + 1)[:, None, None]
    cols = a["BoundaryPoints2D"][1:nj + 1, 1:ni + 1] == 1
    sel = cols[None] & (kk >= np.abs(a["KFloorZ"][1:nj + 1, 1:ni + 1])[None]) & (a["OpenPoints3D"][c] == 1)
    tdec = 1.0 / (1.0 + decay_time / DT)
    ext = P_old[c] * (1.0 - tdec) + ref[c] * tdec
    gain = np.where(w < 0.0, -w * DT * ext, -w * DT * P_new[c])
    if gross:
        return float(np.sum(gain[sel])), float(np.sum(np.abs(gain[sel])))
    return float(np.sum(gain[sel]))


def noflux_masks(d, frac=0.3, seed=0):
    """Seeded NoFluxU/V/W masks (int32, Size box) over a fraction of the compute faces."""
    rng = np.random.default_rng(seed)
    out = []
    for n in ("ComputeFacesU3D", "ComputeFacesV3D", "ComputeFacesW3D"):
        cf = d.arrays[n]
        out.append(((cf == 1) & (rng.random(cf.shape) < frac)).astype(np.int32))
    return tuple(out)


def discharges(d, seed=0, ndis=4, uniform=True, ignore_one=True):
    """Seeded SetDischarges arguments over water columns: point discharges at a
    layer, uniform ones over a layer range or the whole column (Kmin / Kmax not
    given), inflows and withdrawals, a bypass, and an ignored discharge."""
    rng = np.random.default_rng(seed)
    a = d.arrays
    cols = [(j, i) for j in range(1, d.nj + 1) for i in range(1, d.ni + 1)
            if a["WaterPoints3D"][d.nk, j, i] == 1]
    nCells, ignore, bypass, vert = [], [], [], []
    I, J, K, Kmin, Kmax, Flow, Conc, CMF = ([] for _ in range(8))
    for dis in range(ndis):
        nc = int(rng.integers(1, 3))
        ign = 1 if (ignore_one and dis == 1) else 0
        nCells.append(nc)
        ignore.append(ign)
        bypass.append(1 if dis == 2 else 0)
        vert.append(5 if (uniform and dis % 2 == 0) else 1)
        if ign:
            continue                         # the cells of an ignored discharge are not listed
        for _ in range(nc):
            j, i = cols[int(rng.integers(len(cols)))]
            kf = int(a["KFloorZ"][j, i])
            I.append(i)
            J.append(j)
            K.append(int(rng.integers(kf, d.nk + 1)))
            if dis == 0:
                Kmin.append(-9999999)
                Kmax.append(-9999999)
            else:
                k0 = int(rng.integers(kf, d.nk + 1))
                Kmin.append(k0)
                Kmax.append(int(rng.integers(k0, d.nk + 1)))
            Flow.append(float(rng.uniform(-2.0, 6.0)))
            Conc.append(float(rng.uniform(0.5, 8.0)))
            CMF.append(float(rng.uniform(0.5, 1.5)))
    return dict(nCells=np.array(nCells), ignore=np.array(ignore), bypass=np.array(bypass), vert=np.array(vert),
                I=np.array(I), J=np.array(J), K=np.array(K), Kmin=np.array(Kmin), Kmax=np.array(Kmax),
                Flow=np.array(Flow), Conc=np.array(Conc), ConcMF=np.array(CMF))


def fp16_round_fields(d, storage):
    """Round the domain's transports (and, with FP16_QK storage, Visc_H and
    Diff_V) in place to what the batched form stores: FP16 times a per-field
    FP32 scale absmax / 16384.  The oracle then runs on the same inputs as the
    batched kernel, so a comparison measures the arithmetic alone."""
    a = d.arrays
    names = ["Wflux_X", "Wflux_Y", "Wflux_Z"] + (["Visc_H", "Diff_V"] if storage == 2 else [])
    for n in names:
        m = float(np.abs(a[n]).max())
        s = np.float32(m / 16384.0) if m > 0 else np.float32(1.0)
        q = (a[n] * np.float64(np.float32(1.0) / s)).astype(np.float32).astype(np.float16)
        a[n][...] = (s * q.astype(np.float32)).astype(np.float64)
