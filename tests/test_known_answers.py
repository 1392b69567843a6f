"""Known answers independent of the reference's restatement.

Advection at Courant number 1 shifts a field by exactly one cell per step.

On a single layer with V = VolumeZOld = 1, DT = 1, no diffusion and a
transport of +1 (or -1) on every compute face of one direction, the explicit
update of a cell is TI = P + F_in - F_out with F = Q * P_upwind, so a cell
with compute faces on both sides takes its upstream neighbour's value; a cell
against the upstream wall empties and the one against the downstream wall
keeps its value plus the inflow.  With P2_TVD the weight 0.5 * psi * (1 - Cr)
is 0 at Cr = +1, so every limiter gives the same shift for positive
transports (for negative ones the reference's signed Courant number gives
0.5 * psi * 2, which is not a shift; those run with upwind only).

Horizontal diffusion with unit metrics (DUX = DVY = DZX = DZY = AreaU = AreaV
= Visc_H = V = 1, Schmidt 1) and DT = 1/4 is the discrete Laplacian: Kx = 1
(Convert_Visc_Dif_Horizontal's distance-weighted mean of equal viscosities),
each compute face moves (P_neighbour - P) / 4 into the cell.

Implicit horizontal advection at Courant number 1 is a recurrence down each
line (2 x - x_upstream = P between compute faces), exact in dyadic values.
Implicit upwind vertical advection at Courant number 1 is the same recurrence
up a column; explicit vertical advection (upwind or P2_TVD) shifts the column
up one layer, and explicit vertical diffusion through one face with
a = 1/4 exchanges a (P5 - P4).  Vertical diffusion through a single face of a column is a 2 x 2
system whose sum is kept and whose difference shrinks by 1 / (1 + 2 a).

With open boundary columns at both ends of a Courant-1 channel and DecayTime
0, MassConservation makes the inflow cell take its reference and the outflow
cell (P + P_west) / 2, and ImposedValue makes every boundary cell its
reference; a DecayTime blends the inflow's exterior value by 1 / (1 +
DecayTime / DT); Cyclic keeps the boundary rows in the solve, then gives them
their references and copies the interior next to the opposite end;
MassConservNullGrad makes the inflow cell the mean of its old neighbours
across compute faces; NullGradient, with boundary points that do not
neighbour one another, the mean of its neighbours' new values.  In a still layer with Q * DT / V = 1 a point inflow adds its
concentration, a withdrawal with ConcMF = 1 leaves half, and a bypassed
withdrawal adds Q * DT / V * Conc.  NoFlux masks take their faces out of
both answers; the cell fluxes of the two first answers are the upstream value
(advection) and -(P - P_west) (diffusion) on each compute face.

CentralDif and LeapFrog take the face value (P_west + P) / 2 at Courant
number 1.  AdvectionNudging scales each cell's advective terms by
n = min(d_i, d_j, nCells) / nCells on grids at least 2 nCells wide, d the
distance in cells to the nearer edge.

Integer values keep every operation exact (the vertical diffusion case to a
few ulps).
"""
import numpy as np
import pytest

from mohid_gb300 import advdiff, batched
from oracle import oracle as O
from tests.cases import domain

SCHEMES = {
    "upwind1": dict(),
    "tvd_minmod": dict(AdvMethodH=4, TVDLimitationH=1, Upwind2H=1),
    "tvd_vanleer": dict(AdvMethodH=4, TVDLimitationH=2, Upwind2H=1),
    "tvd_muscl": dict(AdvMethodH=4, TVDLimitationH=3, Upwind2H=1),
    "tvd_superbee": dict(AdvMethodH=4, TVDLimitationH=4, Upwind2H=1),
    "tvd_pdm": dict(AdvMethodH=4, TVDLimitationH=5, Upwind2H=1),
}
CASES = [(ax, q, s) for ax in ("j", "i") for q in (1.0, -1.0) for s in SCHEMES if q > 0 or s == "upwind1"]


def channel(axis, q):
    """The single-layer test grid as a uniform channel along j (Wflux_X) or i
    (Wflux_Y) with transport q on every compute face of that direction."""
    d = domain("layer1", dt=1.0)
    a = d.arrays
    for n in ("Wflux_X", "Wflux_Y", "Wflux_Z", "Visc_H", "Diff_V"):
        a[n][...] = 0.0
    a["VolumeZ"][...] = 1.0
    a["VolumeZOld"][...] = 1.0
    name, cf = ("Wflux_X", "ComputeFacesU3D") if axis == "j" else ("Wflux_Y", "ComputeFacesV3D")
    a[name][...] = np.where(a[cf] == 1, q, 0.0)
    P = np.zeros(d.shape3)
    rng = np.random.default_rng(5)
    P[1, 1:d.nj + 1, 1:d.ni + 1] = rng.integers(0, 64, size=(d.nj, d.ni)).astype(np.float64)
    return d, P


def shifted(d, P, axis, q):
    """The closed-form result of one step (work-box cells of the layer)."""
    a = d.arrays
    cf = a["ComputeFacesU3D" if axis == "j" else "ComputeFacesV3D"][1]
    L = P[1]
    out = L.copy()
    for j in range(1, d.nj + 1):
        for i in range(1, d.ni + 1):
            if axis == "j":
                w, e, pw, pe = cf[j, i], cf[j + 1, i], L[j - 1, i], L[j + 1, i]
            else:
                w, e, pw, pe = cf[j, i], cf[j, i + 1], L[j, i - 1], L[j, i + 1]
            p = L[j, i]
            if q > 0:
                out[j, i] = p * (1 - e) + pw * w if (w or e) else p
            else:
                out[j, i] = p * (1 - w) + pe * e if (w or e) else p
    return out[1:d.nj + 1, 1:d.ni + 1]


def params(s):
    return dict(DTProp=1.0, SchmidtBackground_V=0.0, **SCHEMES[s])


@pytest.mark.parametrize("axis,q,scheme", CASES)
def test_oracle_shifts_one_cell(axis, q, scheme):
    d, P = channel(axis, q)
    want = shifted(d, P, axis, q)
    assert not np.array_equal(want, P[1, 1:d.nj + 1, 1:d.ni + 1])      # the field moves
    Q = P.copy()
    assert O.step(d, Q, O.params(**params(scheme))) == 0
    assert np.array_equal(Q[1, 1:d.nj + 1, 1:d.ni + 1], want)


@pytest.mark.gpu
@pytest.mark.parametrize("axis,q,scheme", CASES)
def test_gpu_forms_shift_one_cell(gpu, axis, q, scheme):
    d, P = channel(axis, q)
    want = shifted(d, P, axis, q)
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    Pg = P.copy()
    ad.step(Pg, advdiff.params(**params(scheme)))                     # FP64 drop-in: exact
    assert np.array_equal(Pg[1, 1:d.nj + 1, 1:d.ni + 1], want)
    b = batched.Batch(ad, 1)
    b.set_tracer(0, P)
    b.step(advdiff.params(**params(scheme)))
    b.sync()
    got = b.get_tracer(0)[1, 1:d.nj + 1, 1:d.ni + 1]
    b.destroy()
    ad.kill()
    assert np.max(np.abs(got - want)) <= 1e-6 * np.max(np.abs(want))  # FP32 form


def unit_grid():
    """The single-layer test grid with unit metrics, no transport and unit
    viscosity, and an integer field."""
    d = domain("layer1", dt=0.25)
    a = d.arrays
    for n in ("Wflux_X", "Wflux_Y", "Wflux_Z", "Diff_V"):
        a[n][...] = 0.0
    for n in ("DUX", "DVY", "DZX", "DZY", "AreaU", "AreaV", "Visc_H", "VolumeZ", "VolumeZOld"):
        a[n][...] = 1.0
    P = np.zeros(d.shape3)
    rng = np.random.default_rng(9)
    P[1, 1:d.nj + 1, 1:d.ni + 1] = rng.integers(0, 64, size=(d.nj, d.ni)).astype(np.float64)
    return d, P


def laplacian_step(d, P):
    a = d.arrays
    cu, cv, L = a["ComputeFacesU3D"][1], a["ComputeFacesV3D"][1], P[1]
    out = np.empty((d.nj, d.ni))
    for j in range(1, d.nj + 1):
        for i in range(1, d.ni + 1):
            p = L[j, i]
            out[j - 1, i - 1] = p + 0.25 * (cu[j, i] * (L[j - 1, i] - p) + cu[j + 1, i] * (L[j + 1, i] - p) +
                                            cv[j, i] * (L[j, i - 1] - p) + cv[j, i + 1] * (L[j, i + 1] - p))
    return out


DIFF = dict(DTProp=0.25, SchmidtBackground_V=0.0)


def test_oracle_diffuses_by_the_laplacian():
    d, P = unit_grid()
    want = laplacian_step(d, P)
    assert not np.array_equal(want, P[1, 1:d.nj + 1, 1:d.ni + 1])
    Q = P.copy()
    assert O.step(d, Q, O.params(**DIFF)) == 0
    assert np.array_equal(Q[1, 1:d.nj + 1, 1:d.ni + 1], want)


@pytest.mark.gpu
def test_gpu_forms_diffuse_by_the_laplacian(gpu):
    d, P = unit_grid()
    want = laplacian_step(d, P)
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    Pg = P.copy()
    ad.step(Pg, advdiff.params(**DIFF))
    assert np.array_equal(Pg[1, 1:d.nj + 1, 1:d.ni + 1], want)
    b = batched.Batch(ad, 1)
    b.set_tracer(0, P)
    b.step(advdiff.params(**DIFF))
    b.sync()
    got = b.get_tracer(0)[1, 1:d.nj + 1, 1:d.ni + 1]
    b.destroy()
    ad.kill()
    assert np.max(np.abs(got - want)) <= 1e-6 * np.max(np.abs(want))


@pytest.mark.parametrize("axis", ["j", "i"])
def test_oracle_implicit_advection_recurrence(axis):
    # ImpExp_AdvXX (YY) = 1 at Courant number 1: along each line the implicit
    # upwind rows are 2 x - x_upstream = P between two compute faces, x = P / 2
    # against the upstream wall (outflow only) and x - x_upstream = P against
    # the downstream wall (inflow only), solved by THOMAS_3D along the line
    d, P = channel(axis, 1.0)
    a = d.arrays
    cf = a["ComputeFacesU3D" if axis == "j" else "ComputeFacesV3D"][1]
    L = P[1]
    want = L.copy()
    if axis == "j":
        for i in range(1, d.ni + 1):
            x = 0.0
            for j in range(1, d.nj + 1):
                w, e = cf[j, i], cf[j + 1, i]
                x = (L[j, i] + w * x) / (1.0 + e)
                want[j, i] = x
    else:
        for j in range(1, d.nj + 1):
            x = 0.0
            for i in range(1, d.ni + 1):
                w, e = cf[j, i], cf[j, i + 1]
                x = (L[j, i] + w * x) / (1.0 + e)
                want[j, i] = x
    Q = P.copy()
    imp = dict(ImpExp_AdvXX=1.0) if axis == "j" else dict(ImpExp_AdvYY=1.0)
    assert O.step(d, Q, O.params(DTProp=1.0, SchmidtBackground_V=0.0, **imp)) == 0
    assert np.array_equal(Q[1, 1:d.nj + 1, 1:d.ni + 1], want[1:d.nj + 1, 1:d.ni + 1])


@pytest.mark.parametrize("theta,dt", [(1.0, 1.0), (0.5, 1.0), (0.5, 0.25)])
def test_oracle_vertical_diffusion_through_one_face(theta, dt):
    # a column whose only diffusive face is the one between layers 4 and 5,
    # a = Kz * DUX * DVY / DZZ * DT / V = DT, implicit weight theta
    # (ImpExp_DifV): the two cells solve
    # [[1 + a theta, -a theta], [-a theta, 1 + a theta]] x = P + a (1 - theta) (P5 - P4) (-1, +1),
    # so their sum is kept and their difference scales by
    # (1 - 2 a (1 - theta)) / (1 + 2 a theta); every other layer keeps its
    # value (THOMASZ rounds the divisions, so the pair agrees to a few ulps)
    d = domain("column", dt=dt)
    a = d.arrays
    for n in ("Wflux_X", "Wflux_Y", "Wflux_Z", "Visc_H", "Diff_V"):
        a[n][...] = 0.0
    for n in ("DUX", "DVY", "DZZ", "VolumeZ", "VolumeZOld"):
        a[n][...] = 1.0
    a["ComputeFacesW3D"][...] = 0                  # a lone column has none of its own
    a["ComputeFacesW3D"][5, 1, 1] = 1
    a["Diff_V"][5, 1, 1] = 1.0
    P = np.zeros(d.shape3)
    P[1:d.nk + 1, 1, 1] = np.arange(1, d.nk + 1, dtype=np.float64) * 8.0
    Q = P.copy()
    assert O.step(d, Q, O.params(DTProp=dt, SchmidtBackground_V=0.0, SchmidtCoef_V=1.0, ImpExp_DifV=theta)) == 0
    p4, p5 = P[4, 1, 1], P[5, 1, 1]
    x4, x5 = Q[4, 1, 1], Q[5, 1, 1]
    a_ = dt
    assert abs((x4 + x5) - (p4 + p5)) <= 4 * np.spacing(p4 + p5)
    want = (p4 - p5) * (1.0 - 2.0 * a_ * (1.0 - theta)) / (1.0 + 2.0 * a_ * theta)
    assert abs((x4 - x5) - want) <= 8 * np.spacing(p4 + p5)
    others = [k for k in range(1, d.nk + 1) if k not in (4, 5)]
    assert np.array_equal(Q[others, 1, 1], P[others, 1, 1])


@pytest.mark.parametrize("docycle", [1, 2])
def test_oracle_implicit_vertical_advection_recurrence(docycle):
    # upward transport 1 through every interior face of a column (V = 1,
    # DT = 1, closed surface, no diffusion): implicit upwind rows are
    # 2 x - x_below = P, x = P / 2 at the bed (outflow only) and
    # x - x_below = P at the top (inflow only); THOMASZ solves them exactly
    d = domain("column", dt=1.0)
    a = d.arrays
    nk = d.nk
    for n in ("Wflux_X", "Wflux_Y", "Wflux_Z", "Visc_H", "Diff_V"):
        a[n][...] = 0.0
    for n in ("DUX", "DVY", "DZZ", "DWZ", "VolumeZ", "VolumeZOld"):
        a[n][...] = 1.0
    a["OpenPoints3D"][...] = 0
    a["OpenPoints3D"][1:nk + 1, 1, 1] = 1
    a["ComputeFacesW3D"][...] = 0
    a["ComputeFacesW3D"][2:nk + 1, 1, 1] = 1
    a["Wflux_Z"][2:nk + 1, 1, 1] = 1.0
    P = np.zeros(d.shape3)
    P[1:nk + 1, 1, 1] = np.random.default_rng(3).integers(0, 64, size=nk).astype(np.float64)
    want = np.empty(nk)
    x = 0.0
    for k in range(1, nk + 1):
        inflow = 1.0 if k > 1 else 0.0
        outflow = 1.0 if k < nk else 0.0
        x = (P[k, 1, 1] + inflow * x) / (1.0 + outflow)
        want[k - 1] = x
    Q = P.copy()
    assert O.step(d, Q, O.params(DTProp=1.0, SchmidtBackground_V=0.0, Docycle_method=docycle)) == 0
    assert np.array_equal(Q[1:nk + 1, 1, 1], want)


def open_channel():
    """The Courant-1 channel along j with the columns at j = 1 and j = JUB
    marked as boundary points, and an integer reference field."""
    d, P = channel("j", 1.0)
    a = d.arrays
    a["BoundaryPoints2D"][...] = 0
    a["BoundaryPoints2D"][1, 1:d.ni + 1] = 1
    a["BoundaryPoints2D"][d.nj, 1:d.ni + 1] = 1
    R = np.zeros(d.shape3)
    R[1, 1:d.nj + 1, 1:d.ni + 1] = np.random.default_rng(11).integers(0, 64, size=(d.nj, d.ni)).astype(np.float64)
    return d, P, R


@pytest.mark.parametrize("scheme", ["upwind1", "tvd_superbee"])
def test_oracle_mass_conservation_boundary_feeds_the_channel(scheme):
    # MassConservation, DecayTime 0: the inflow cell (j = 1) empties through
    # its east face and takes -WFOB * DT * Ref = Ref; the outflow cell (j = JUB)
    # gains its west neighbour and loses WFOB * DT * x implicitly, so
    # x = (P + P_west) / 2; the interior shifts by one cell
    d, P, R = open_channel()
    L, nj = P[1], d.nj
    want = L.copy()
    want[2:nj, :] = L[1:nj - 1, :]
    want[1, :] = R[1, 1, :]
    want[nj, :] = (L[nj, :] + L[nj - 1, :]) / 2.0
    Q = P.copy()
    assert O.step(d, Q, O.params(BoundaryCondition=1, **params(scheme)), ReferenceProp=R) == 0
    assert np.array_equal(Q[1, 1:nj + 1, 1:d.ni + 1], want[1:nj + 1, 1:d.ni + 1])


@pytest.mark.parametrize("bc", [2, 5])
def test_oracle_imposed_value_boundary_takes_the_reference(bc):
    # ImposedValue (2) and SubModel (5), DecayTime 0: the boundary cells are
    # identity rows with the interior mean decayed fully towards the reference
    # (decay factor 1), whatever the interior does
    d, P, R = open_channel()
    Q = P.copy()
    assert O.step(d, Q, O.params(BoundaryCondition=bc, **params("upwind1")), ReferenceProp=R) == 0
    for j in (1, d.nj):
        assert np.array_equal(Q[1, j, 1:d.ni + 1], R[1, j, 1:d.ni + 1])


@pytest.mark.parametrize("decay,tdec", [(1.0, 0.5), (3.0, 0.25)])
def test_oracle_boundary_decay_blends_the_inflow(decay, tdec):
    # MassConservation with DecayTime: the inflow carries the exterior value
    # P * (1 - tdec) + Ref * tdec, tdec = 1 / (1 + DecayTime / DT)
    d, P, R = open_channel()
    Q = P.copy()
    assert O.step(d, Q, O.params(BoundaryCondition=1, DecayTime=decay, **params("upwind1")), ReferenceProp=R) == 0
    want = P[1, 1, 1:d.ni + 1] * (1.0 - tdec) + R[1, 1, 1:d.ni + 1] * tdec
    assert np.array_equal(Q[1, 1, 1:d.ni + 1], want)


def test_oracle_discharges_add_and_withdraw():
    # a still layer (V = VolumeZOld = 1, DT = 1, no transport or diffusion):
    # a point inflow of Q = 1 adds Q * DT / V * Conc to its cell, a withdrawal
    # of Q = -1 with ConcMF = 1 leaves implicitly (E = 1 + 1: half remains), a
    # bypassed withdrawal adds Q * DT / V * Conc like an inflow
    d = domain("layer1", dt=1.0)
    a = d.arrays
    for n in ("Wflux_X", "Wflux_Y", "Wflux_Z", "Visc_H", "Diff_V"):
        a[n][...] = 0.0
    a["VolumeZ"][...] = 1.0
    a["VolumeZOld"][...] = 1.0
    P = np.zeros(d.shape3)
    P[1, 1:d.nj + 1, 1:d.ni + 1] = np.random.default_rng(13).integers(0, 64, size=(d.nj, d.ni)).astype(np.float64)
    cells = [(2, 3), (4, 5), (6, 2)]                   # (j, i): inflow, withdrawal, bypassed withdrawal
    ds = dict(nCells=np.array([1, 1, 1]), ignore=np.array([0, 0, 0]), bypass=np.array([0, 0, 1]),
              vert=np.array([1, 1, 1]), I=np.array([c[1] for c in cells]), J=np.array([c[0] for c in cells]),
              K=np.array([1, 1, 1]), Kmin=np.array([-9999999] * 3), Kmax=np.array([-9999999] * 3),
              Flow=np.array([1.0, -1.0, -1.0]), Conc=np.array([5.0, 7.0, 3.0]), ConcMF=np.array([2.0, 1.0, 4.0]))
    want = P[1].copy()
    want[2, 3] += 5.0
    want[4, 5] /= 2.0
    want[6, 2] += -1.0 * 3.0
    Q = P.copy()
    assert O.step(d, Q, O.params(DTProp=1.0, SchmidtBackground_V=0.0), Disch=ds) == 0
    assert np.array_equal(Q[1, 1:d.nj + 1, 1:d.ni + 1], want[1:d.nj + 1, 1:d.ni + 1])


def test_oracle_noflux_masks_stop_the_shift_and_the_laplacian():
    # NoAdvFlux / NoDifFlux: a masked face carries nothing, so the known
    # answers hold with the masked faces taken out of the compute faces
    d, P = channel("j", 1.0)
    a = d.arrays
    rng = np.random.default_rng(17)
    nfu = ((a["ComputeFacesU3D"] == 1) & (rng.random(a["ComputeFacesU3D"].shape) < 0.3)).astype(np.int32)
    zero = np.zeros_like(nfu)
    nf = (nfu, zero, zero)
    cfu = a["ComputeFacesU3D"].copy()
    a["ComputeFacesU3D"][...] = cfu * (1 - nfu)            # the faces that still carry flux
    want = shifted(d, P, "j", 1.0)
    a["ComputeFacesU3D"][...] = cfu
    Q = P.copy()
    assert O.step(d, Q, O.params(NoAdvFlux=1, **params("upwind1")), NoFlux=nf) == 0
    assert np.array_equal(Q[1, 1:d.nj + 1, 1:d.ni + 1], want)

    d, P = unit_grid()
    a = d.arrays
    nfu = ((a["ComputeFacesU3D"] == 1) & (rng.random(a["ComputeFacesU3D"].shape) < 0.3)).astype(np.int32)
    nfv = ((a["ComputeFacesV3D"] == 1) & (rng.random(a["ComputeFacesV3D"].shape) < 0.3)).astype(np.int32)
    cfu, cfv = a["ComputeFacesU3D"].copy(), a["ComputeFacesV3D"].copy()
    a["ComputeFacesU3D"][...] = cfu * (1 - nfu)
    a["ComputeFacesV3D"][...] = cfv * (1 - nfv)
    want = laplacian_step(d, P)
    a["ComputeFacesU3D"][...] = cfu
    a["ComputeFacesV3D"][...] = cfv
    Q = P.copy()
    assert O.step(d, Q, O.params(NoDifFlux=1, **DIFF), NoFlux=(nfu, nfv, np.zeros_like(nfu))) == 0
    assert np.array_equal(Q[1, 1:d.nj + 1, 1:d.ni + 1], want)


def test_oracle_cell_fluxes_of_the_known_steps():
    # CellFluxes (GetAdvFlux / GetDifFlux): at Courant number 1 the advective
    # flux through a compute face is the upstream value; with unit metrics the
    # diffusive flux through a west face is -(P - P_west)
    d, P = channel("j", 1.0)
    work = O.Work(d)
    Q = P.copy()
    assert O.step(d, Q, O.params(CellFluxes=1, **params("upwind1")), work=work) == 0
    f = O.cell_fluxes(d, work)
    cf = d.arrays["ComputeFacesU3D"][1]
    L = P[1]
    want = np.zeros_like(L)
    want[1:, :] = cf[1:, :] * L[:-1, :]
    assert np.array_equal(f["AdvFluxX"][1], want)
    assert not f["DifFluxX"].any() and not f["AdvFluxY"].any()

    d, P = unit_grid()
    work = O.Work(d)
    Q = P.copy()
    assert O.step(d, Q, O.params(CellFluxes=1, **DIFF), work=work) == 0
    f = O.cell_fluxes(d, work)
    cf = d.arrays["ComputeFacesU3D"][1]
    L = P[1]
    want = np.zeros_like(L)
    want[1:, :] = -cf[1:, :] * (L[1:, :] - L[:-1, :])
    assert np.array_equal(f["DifFluxX"][1], want)
    assert not f["AdvFluxX"].any()


def test_oracle_cyclic_boundaries_copy_across_the_channel():
    # Cyclic: the boundary rows keep their old values in the solve (the
    # interior shifts, taking the old j = 1 value into j = 2); after it every
    # boundary cell takes its reference, then each row i = 2..IUB-1 whose two
    # ends are boundary points copies the interior next to the opposite end
    d, P, R = open_channel()
    L, nj, ni = P[1], d.nj, d.ni
    new = L.copy()
    new[2:nj, :] = L[1:nj - 1, :]                    # the interior's Courant-1 shift
    want = new.copy()
    want[1, :] = R[1, 1, :]
    want[nj, :] = R[1, nj, :]
    for i in range(2, ni):
        want[1, i] = new[nj - 1, i]
        want[nj, i] = new[2, i]
    Q = P.copy()
    assert O.step(d, Q, O.params(BoundaryCondition=8, **params("upwind1")), ReferenceProp=R) == 0
    assert np.array_equal(Q[1, 1:nj + 1, 1:ni + 1], want[1:nj + 1, 1:ni + 1])


def _case(name):
    """(domain, field, params, ReferenceProp, discharges, NoFlux masks,
    batched form takes it) of the known-answer cases run on the GPU forms."""
    R = ds = nf = None
    if name == "implicit_j":
        d, P = channel("j", 1.0)
        pd = dict(params("upwind1"), ImpExp_AdvXX=1.0)
        return d, P, pd, R, ds, nf, False
    if name in ("mass_conservation", "imposed_value", "cyclic", "decay"):
        d, P, R = open_channel()
        bc = {"mass_conservation": 1, "imposed_value": 2, "cyclic": 8, "decay": 1}[name]
        pd = dict(params("tvd_superbee"), BoundaryCondition=bc, DecayTime=3.0 if name == "decay" else 0.0)
        return d, P, pd, R, ds, nf, True
    if name == "discharges":
        d = domain("layer1", dt=1.0)
        a = d.arrays
        for n in ("Wflux_X", "Wflux_Y", "Wflux_Z", "Visc_H", "Diff_V"):
            a[n][...] = 0.0
        a["VolumeZ"][...] = 1.0
        a["VolumeZOld"][...] = 1.0
        P = np.zeros(d.shape3)
        P[1, 1:d.nj + 1, 1:d.ni + 1] = np.random.default_rng(13).integers(0, 64, size=(d.nj, d.ni)).astype(float)
        ds = dict(nCells=np.array([1, 1, 1]), ignore=np.array([0, 0, 0]), bypass=np.array([0, 0, 1]),
                  vert=np.array([1, 1, 1]), I=np.array([3, 5, 2]), J=np.array([2, 4, 6]), K=np.array([1, 1, 1]),
                  Kmin=np.array([-9999999] * 3), Kmax=np.array([-9999999] * 3),
                  Flow=np.array([1.0, -1.0, -1.0]), Conc=np.array([5.0, 7.0, 3.0]), ConcMF=np.array([2.0, 1.0, 4.0]))
        return d, P, dict(DTProp=1.0, SchmidtBackground_V=0.0), R, ds, nf, True
    if name in ("noflux_adv", "noflux_dif"):
        d, P = channel("j", 1.0) if name == "noflux_adv" else unit_grid()
        a = d.arrays
        rng = np.random.default_rng(17)
        nfu = ((a["ComputeFacesU3D"] == 1) & (rng.random(a["ComputeFacesU3D"].shape) < 0.3)).astype(np.int32)
        nfv = ((a["ComputeFacesV3D"] == 1) & (rng.random(a["ComputeFacesV3D"].shape) < 0.3)).astype(np.int32)
        nf = (nfu, nfv, np.zeros_like(nfu))
        pd = dict(params("upwind1"), NoAdvFlux=1) if name == "noflux_adv" else dict(DIFF, NoDifFlux=1)
        return d, P, pd, R, ds, nf, True
    raise ValueError(name)


GPU_CASES = ["implicit_j", "mass_conservation", "imposed_value", "cyclic", "decay", "discharges", "noflux_adv",
             "noflux_dif"]


def _oracle(name):
    d, P, pd, R, ds, nf, _ = _case(name)
    Q = P.copy()
    assert O.step(d, Q, O.params(**pd), ReferenceProp=R, Disch=ds, NoFlux=nf) == 0
    return Q


@pytest.mark.parametrize("name", GPU_CASES)
def test_known_answer_cases_build(name):
    # the cases the GPU test below runs, on the oracle
    Q = _oracle(name)
    assert np.isfinite(Q).all()


@pytest.mark.gpu
@pytest.mark.parametrize("name", GPU_CASES)
def test_gpu_forms_on_the_known_answer_cases(gpu, name):
    # the FP64 drop-in equals the oracle bit for bit on every case (whose
    # closed forms the CPU tests above pin); the batched form, where it takes
    # the options, to 1e-6
    d, P, pd, R, ds, nf, batch_ok = _case(name)
    want = _oracle(name)
    ad = advdiff.AdvectionDiffusion(d)
    ad.set_hydro()
    if nf is not None:
        ad.set_noflux(nf)
    if ds is not None:
        ad.set_discharges(ds)
    Pg = P.copy()
    ad.step(Pg, advdiff.params(**pd), R)
    assert np.array_equal(Pg, want)
    if batch_ok:
        b = batched.Batch(ad, 1)
        b.set_tracer(0, P)
        if ds is not None:
            b.set_discharge_conc(0, ds["Conc"])
        if R is not None:
            b.set_reference(0, R)
        b.step(advdiff.params(**pd))
        b.sync()
        got = b.get_tracer(0)
        b.destroy()
        c = (1, slice(1, d.nj + 1), slice(1, d.ni + 1))
        assert np.max(np.abs(got[c] - want[c])) <= 1e-6 * np.max(np.abs(want[c]))
    ad.kill()


@pytest.mark.parametrize("name", GPU_CASES + ["shift_j", "shift_i_neg", "laplacian"])
def test_python_restatement_on_the_known_answer_cases(name):
    # the second, pure-Python restatement gives the oracle's bits on the
    # closed-form cases too (so both reproduce the closed forms)
    from oracle import ref_py
    if name == "shift_j":
        (d, P), pd, R, ds, nf = channel("j", 1.0), params("tvd_superbee"), None, None, None
    elif name == "shift_i_neg":
        (d, P), pd, R, ds, nf = channel("i", -1.0), params("upwind1"), None, None, None
    elif name == "laplacian":
        (d, P), pd, R, ds, nf = unit_grid(), DIFF, None, None, None
    else:
        d, P, pd, R, ds, nf, _ = _case(name)
    Q = P.copy()
    assert O.step(d, Q, O.params(**pd), ReferenceProp=R, Disch=ds, NoFlux=nf) == 0
    Pp = P.copy()
    ref_py.step(d, Pp, dict(O.DEFAULTS, **pd), ReferenceProp=R, Disch=ds, NoFlux=nf)
    assert np.array_equal(Pp, Q)


def test_oracle_nudging_scales_the_shift():
    # AdvectionNudging with nCells = 2 on the 6 x 7 layer (at least 2 nCells
    # wide, so the reference's in-order distances are the distances to the
    # nearer edge): each cell's advective terms enter scaled by
    # n = min(d_i, d_j, nCells) / nCells, so at Courant number 1 a cell gets
    # P + n * (P_west * w - P * e)
    d, P = channel("j", 1.0)
    nc = 2
    cf = d.arrays["ComputeFacesU3D"][1]
    L = P[1]
    want = L.copy()
    for j in range(1, d.nj + 1):
        for i in range(1, d.ni + 1):
            di, dj = min(i, d.ni - i + 1), min(j, d.nj - j + 1)
            n = min(di, dj, nc) / nc
            want[j, i] = L[j, i] + n * (L[j - 1, i] * cf[j, i] - L[j, i] * cf[j + 1, i])
    pd = dict(params("upwind1"), AdvectionNudging=1, AdvectionNudgingCells=nc)
    Q = P.copy()
    assert O.step(d, Q, O.params(**pd)) == 0
    assert np.array_equal(Q[1, 1:d.nj + 1, 1:d.ni + 1], want[1:d.nj + 1, 1:d.ni + 1])
    from oracle import ref_py
    Pp = P.copy()
    ref_py.step(d, Pp, dict(O.DEFAULTS, **pd))
    assert np.array_equal(Pp, Q)


@pytest.mark.parametrize("method", [5, 6])
def test_oracle_central_face_at_courant_one(method):
    # CentralDif (5) and LeapFrog (6) take the face value (P_west + P) / 2 at
    # Courant number 1, so a cell gets P + w (P_west + P) / 2 - e (P + P_east) / 2
    d, P = channel("j", 1.0)
    cf = d.arrays["ComputeFacesU3D"][1]
    L = P[1]
    want = L.copy()
    for j in range(1, d.nj + 1):
        for i in range(1, d.ni + 1):
            want[j, i] = L[j, i] + cf[j, i] * 0.5 * (L[j - 1, i] + L[j, i]) - \
                cf[j + 1, i] * 0.5 * (L[j, i] + L[j + 1, i])
    Q = P.copy()
    assert O.step(d, Q, O.params(DTProp=1.0, SchmidtBackground_V=0.0, AdvMethodH=method)) == 0
    assert np.array_equal(Q[1, 1:d.nj + 1, 1:d.ni + 1], want[1:d.nj + 1, 1:d.ni + 1])


def upward_column():
    """A lone column with every interior face a compute face, transport 1
    upward through them (V = 1, DT = 1, closed surface), an integer field."""
    d = domain("column", dt=1.0)
    a = d.arrays
    nk = d.nk
    for n in ("Wflux_X", "Wflux_Y", "Wflux_Z", "Visc_H", "Diff_V"):
        a[n][...] = 0.0
    for n in ("DUX", "DVY", "DZZ", "DWZ", "VolumeZ", "VolumeZOld"):
        a[n][...] = 1.0
    a["OpenPoints3D"][...] = 0
    a["OpenPoints3D"][1:nk + 1, 1, 1] = 1
    a["ComputeFacesW3D"][...] = 0
    a["ComputeFacesW3D"][2:nk + 1, 1, 1] = 1
    a["Wflux_Z"][2:nk + 1, 1, 1] = 1.0
    P = np.zeros(d.shape3)
    P[1:nk + 1, 1, 1] = np.random.default_rng(3).integers(0, 64, size=nk).astype(np.float64)
    return d, P


@pytest.mark.parametrize("vopt", [dict(), dict(AdvMethodV=4, TVDLimitationV=4, Upwind2V=1)])
def test_oracle_explicit_vertical_advection_shifts_up(vopt):
    # ImpExp_AdvV = 0 at Courant number 1: each layer takes the one below; the
    # bed empties, the top keeps its value plus the inflow (P2_TVD's weight
    # vanishes at Cr = 1 as horizontally)
    d, P = upward_column()
    nk = d.nk
    c = P[:, 1, 1]
    want = c.copy()
    want[1] = 0.0
    want[2:nk] = c[1:nk - 1]
    want[nk] = c[nk] + c[nk - 1]
    Q = P.copy()
    assert O.step(d, Q, O.params(DTProp=1.0, SchmidtBackground_V=0.0, ImpExp_AdvV=0.0, **vopt)) == 0
    assert np.array_equal(Q[1:nk + 1, 1, 1], want[1:nk + 1])


def test_oracle_explicit_vertical_diffusion_through_one_face():
    # ImpExp_DifV = 0, one diffusive face between layers 4 and 5 with
    # a = Kz * DUX * DVY / DZZ * DT / V = 1/4: the pair exchanges
    # a * (P5 - P4), the other layers keep their values
    d = domain("column", dt=0.25)
    a = d.arrays
    for n in ("Wflux_X", "Wflux_Y", "Wflux_Z", "Visc_H", "Diff_V"):
        a[n][...] = 0.0
    for n in ("DUX", "DVY", "DZZ", "VolumeZ", "VolumeZOld"):
        a[n][...] = 1.0
    a["ComputeFacesW3D"][...] = 0
    a["ComputeFacesW3D"][5, 1, 1] = 1
    a["Diff_V"][5, 1, 1] = 1.0
    P = np.zeros(d.shape3)
    P[1:d.nk + 1, 1, 1] = np.arange(1, d.nk + 1, dtype=np.float64) * 8.0
    want = P[:, 1, 1].copy()
    flux = 0.25 * (P[5, 1, 1] - P[4, 1, 1])
    want[4] += flux
    want[5] -= flux
    Q = P.copy()
    assert O.step(d, Q, O.params(DTProp=0.25, SchmidtBackground_V=0.0, ImpExp_DifV=0.0)) == 0
    assert np.array_equal(Q[1:d.nk + 1, 1, 1], want[1:d.nk + 1])


def test_oracle_mass_conserv_null_grad_boundary():
    # MassConservNullGrad (7): the inflow cell (j = 1) becomes the mean of its
    # old neighbours across compute faces (east, and north / south along the
    # boundary row where those are compute faces); the outflow cell leaves
    # implicitly as with MassConservation, (P + P_west) / 2
    d, P, R = open_channel()
    a = d.arrays
    cu, cv, L, nj, ni = a["ComputeFacesU3D"][1], a["ComputeFacesV3D"][1], P[1], d.nj, d.ni
    Q = P.copy()
    assert O.step(d, Q, O.params(BoundaryCondition=7, **params("upwind1")), ReferenceProp=R) == 0
    for i in range(1, ni + 1):
        nb = [(cu[2, i], L[2, i]), (cv[1, i + 1], L[1, i + 1]), (cv[1, i], L[1, i - 1])]
        w = sum(c for c, _ in nb)
        mean = sum(c * v for c, v in nb) / w
        assert abs(Q[1, 1, i] - mean) <= 2 * np.spacing(max(abs(mean), 1.0))
    assert np.array_equal(Q[1, nj, 1:ni + 1], (L[nj, 1:ni + 1] + L[nj - 1, 1:ni + 1]) / 2.0)
    assert np.array_equal(Q[1, 2:nj, 1:ni + 1], L[1:nj - 1, 1:ni + 1])


def test_oracle_null_gradient_boundary_mean():
    # NullGradient (4) with boundary points at every other cell of the j = 1
    # row, so that no boundary cell neighbours another and the in-order sweep
    # has no order to depend on: the boundary rows keep their old values in
    # the solve (the east neighbour then holds the boundary cell's old value,
    # shifted in), and each boundary cell becomes the mean of its neighbours'
    # new values across compute faces; the other cells of the row, against the
    # upstream wall, empty
    d, P = channel("j", 1.0)
    a = d.arrays
    a["BoundaryPoints2D"][...] = 0
    a["BoundaryPoints2D"][1, 1:d.ni + 1:2] = 1
    cu, cv, L, ni = a["ComputeFacesU3D"][1], a["ComputeFacesV3D"][1], P[1], d.ni
    Q = P.copy()
    assert O.step(d, Q, O.params(BoundaryCondition=4, **params("upwind1"))) == 0
    new = np.zeros_like(L)
    new[2, :] = L[1, :]                         # the east neighbours: the old boundary-row values
    for i in range(1, ni + 1, 2):
        nb = [(cu[2, i], new[2, i]), (cv[1, i + 1], 0.0), (cv[1, i], 0.0)]   # row neighbours emptied
        w = sum(c for c, _ in nb)
        mean = sum(c * v for c, v in nb) / w
        assert abs(Q[1, 1, i] - mean) <= 2 * np.spacing(max(abs(mean), 1.0))
    for i in range(2, ni + 1, 2):
        assert Q[1, 1, i] == 0.0


def test_oracle_small_depths_skip_vertical_diffusion():
    # a column flagged in SmallDepths takes no vertical diffusion
    # (VerticalDiffusion skips it): the one-face exchange leaves it unchanged
    d = domain("column", dt=1.0)
    a = d.arrays
    for n in ("Wflux_X", "Wflux_Y", "Wflux_Z", "Visc_H", "Diff_V"):
        a[n][...] = 0.0
    for n in ("DUX", "DVY", "DZZ", "VolumeZ", "VolumeZOld"):
        a[n][...] = 1.0
    a["ComputeFacesW3D"][...] = 0
    a["ComputeFacesW3D"][5, 1, 1] = 1
    a["Diff_V"][5, 1, 1] = 1.0
    P = np.zeros(d.shape3)
    P[1:d.nk + 1, 1, 1] = np.arange(1, d.nk + 1, dtype=np.float64) * 8.0
    sd = np.zeros(a["KFloorZ"].shape, dtype=np.int32)
    sd[1, 1] = 1
    Q = P.copy()
    assert O.step(d, Q, O.params(DTProp=1.0, SchmidtBackground_V=0.0), SmallDepths=sd) == 0
    assert np.array_equal(Q[1:d.nk + 1, 1, 1], P[1:d.nk + 1, 1, 1])


@pytest.mark.parametrize("case", ["vertical1d", "xzflow", "nulldif"])
def test_oracle_options_that_stop_the_known_answers(case):
    # Vertical1D drops the horizontal terms (a single layer then keeps its
    # values); XZFlow drops the y direction (a channel along i keeps its
    # values); NullDif zeroes diffusion across faces without transport (the
    # Laplacian grid has none, so it keeps its values)
    if case == "vertical1d":
        (d, P), pd = channel("j", 1.0), dict(params("upwind1"), Vertical1D=1)
    elif case == "xzflow":
        (d, P), pd = channel("i", 1.0), dict(params("upwind1"), XZFlow=1)
    else:
        (d, P), pd = unit_grid(), dict(DIFF, NullDif=1)
    Q = P.copy()
    assert O.step(d, Q, O.params(**pd)) == 0
    assert np.array_equal(Q[1, 1:d.nj + 1, 1:d.ni + 1], P[1, 1:d.nj + 1, 1:d.ni + 1])
