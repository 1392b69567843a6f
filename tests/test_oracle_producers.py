"""The oracle's restatements of the step's producers (ModuleGeometry's
distances, volumes and areas; ModuleHydrodynamic's vertical water flux from
continuity) against known answers:

* the seeded domains are built with MOHID's own geometry and continuity rules,
  so from their layer interfaces the geometry restatement reproduces their
  thicknesses, volumes and face areas, and from their horizontal fluxes the
  vertical-flux restatement reproduces their vertical transport;
* the produced vertical flux closes every water cell's water budget to
  round-off, and a fixed grid equals a variable one when the volumes do not move.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.cases import domain


def szz_from(d):
    """Layer interfaces SZZ (Size box) of a domain: SZZ(KUB) = 0 at the surface,
    SZZ(k-1) = SZZ(k) + DWZ(k) downwards, so that DWZ = SZZ(k-1) - SZZ(k)."""
    dwz = d.arrays["DWZ"]
    szz = np.zeros(d.shape3)
    for k in range(d.nk, 0, -1):
        szz[k - 1] = szz[k] + dwz[k]
    szz[d.nk + 1] = szz[d.nk]
    return szz


def grid_lengths(d):
    """DXX, DYY (2-D Size box) the seeded generator uses for the face areas."""
    dx, dy = d.spec.dx, d.spec.dy
    return np.full(d.shape2, dx), np.full(d.shape2, dy)


@pytest.mark.parametrize("grid", ["coast", "zlevel", "open", "nsopen"])
def test_geometry_reproduces_the_seeded_domains(built, grid):
    d = domain(grid)
    a = d.arrays
    dxx, dyy = grid_lengths(d)
    out = {n: np.zeros(d.shape3) for n in O.GEOMETRY_OUT}
    out["DWZ"][d.nk + 1] = a["DWZ"][d.nk + 1]
    O.geometry(d.ni, d.nj, d.nk, szz_from(d), a["WaterPoints3D"], a["DUX"], a["DVY"], dxx, dyy,
               3, False, out)
    wp = d.water_mask()
    wk = np.zeros(d.shape3, bool)
    wk[1:-1, 1:-1, 1:-1] = True
    # thicknesses of water cells: SZZ differences of the same values
    np.testing.assert_allclose(out["DWZ"][wp], a["DWZ"][wp], rtol=1e-13)
    np.testing.assert_allclose(out["DZZ"][wp & wk], a["DZZ"][wp & wk], rtol=1e-13)
    # volumes: DWZ * DUX * DVY on every work-box cell
    np.testing.assert_allclose(out["VolumeZ"][wk & wp], a["VolumeZOld"][wk & wp], rtol=1e-13)
    # face areas between two water cells: minimum thickness times the face length
    both_u = wp.copy()
    both_u[:, 1:, :] &= wp[:, :-1, :]
    both_u[:, 0, :] = False
    both_u &= wk
    both_u[:, 1, :] = False                         # j = JLB: not computed by the reference
    np.testing.assert_allclose(out["AreaU"][both_u], a["AreaU"][both_u], rtol=1e-13)


@pytest.mark.parametrize("grid", ["coast", "zlevel", "open"])
def test_vertical_flux_reproduces_the_seeded_transport(built, grid):
    d = domain(grid)
    a = d.arrays
    qz = np.zeros(d.shape3)
    O.vertical_flux(d, qz, d.spec.dt, True)
    # open-boundary columns exchange water through their exterior faces, which
    # are not compute faces: the reference's continuity leaves that flow out
    # (it reappears as the boundary flux of the transport step), the seeded
    # transport does not; compare the interior columns
    wp = d.water_mask() & (a["BoundaryPoints2D"] != 1)[None]
    inner = np.zeros(d.shape3, bool)
    inner[1:d.nk + 1] = True                        # faces below each water cell
    sel = wp & inner
    scale = np.abs(a["Wflux_X"]).max() + np.abs(a["Wflux_Y"]).max()
    assert np.max(np.abs(qz[sel] - a["Wflux_Z"][sel])) <= 1e-12 * scale
    # the surface face carries the column's residual: round-off on a closed surface
    top = qz[d.nk + 1][wp[d.nk]]
    assert np.max(np.abs(top)) <= 1e-11 * scale


def test_vertical_flux_closes_each_cell_budget(built):
    d = domain("open")                               # moving volumes
    a = d.arrays
    qz = np.zeros(d.shape3)
    O.vertical_flux(d, qz, d.spec.dt, True)
    nk, nj, ni = d.nk, d.nj, d.ni
    c = (slice(1, nk + 1), slice(1, nj + 1), slice(1, ni + 1))
    qx = a["Wflux_X"] * a["ComputeFacesU3D"]
    qy = a["Wflux_Y"] * a["ComputeFacesV3D"]
    r = (qx[c] - qx[1:nk + 1, 2:nj + 2, 1:ni + 1] + qy[c] - qy[1:nk + 1, 1:nj + 1, 2:ni + 2] +
         qz[c] - qz[2:nk + 2, 1:nj + 1, 1:ni + 1] - (a["VolumeZ"][c] - a["VolumeZOld"][c]) / d.spec.dt)
    wp = d.water_mask()[c]
    assert np.max(np.abs(r[wp])) <= 1e-12 * np.abs(a["Wflux_X"]).max()


def test_fixed_grid_equals_variable_grid_on_static_volumes(built):
    d = domain("coast")
    q1, q2 = np.zeros(d.shape3), np.zeros(d.shape3)
    assert np.array_equal(d.arrays["VolumeZ"], d.arrays["VolumeZOld"])
    O.vertical_flux(d, q1, d.spec.dt, True)
    O.vertical_flux(d, q2, d.spec.dt, False)
    assert np.array_equal(q1, q2)
