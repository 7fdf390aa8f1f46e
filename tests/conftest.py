import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(REPO / "shallow-water-eric_gb300"))
sys.path.insert(0, str(REPO))
GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    return GOLDEN


# The reference's test cases (type_test) on the reference's own meshes where
# they are shipped small (committed gzip copies), else on a jittered mesh of
# the same domain (ARNAU/mesh_0.05 and TIDAL_WAVE_ISLAND/cav_0.5 are large).
# Dirichlet sides follow the cav meshes' numbering: 1 x = 0, 2 y = 1 (top),
# 3 x = x_max, 4 y = 0; walls qx = 0 on 1/3 and qy = 0 on 2/4; the bump flows
# take q at the inflow side 1 and (subcritical outflow) h at side 3.
REF_CASES = {
    1: ("jitter", (41, 21, 0.0, 2.0, 0.0, 1.0, 7), dict(ux_dir=[1, 3], uy_dir=[2, 4], tfinal=1.0)),
    2: ("ref_bump_cav_0.3.FEM.gz", None, dict(ux_dir=[1, 3], uy_dir=[2, 4], tfinal=1.0)),
    3: ("ref_bump_cav_0.3.FEM.gz", None, dict(h_dir=[3], ux_dir=[1], uy_dir=[2, 4], tfinal=1.0)),
    4: ("ref_dam_cav_0.25.FEM.gz", None, dict(ux_dir=[1, 3], uy_dir=[2, 4], tfinal=6.0)),
    6: ("ref_bump_cav_0.3.FEM.gz", None, dict(ux_dir=[1], uy_dir=[2, 4], tfinal=1.0)),
    7: ("ref_bump_cav_0.3.FEM.gz", None, dict(h_dir=[3], ux_dir=[1], uy_dir=[2, 4], tfinal=1.0)),
    8: ("jitter", (61, 51, 0.0, 30.0, 0.0, 25.0, 8), dict(ux_dir=[1, 3], uy_dir=[2, 4], tfinal=1.0)),
    11: ("ref_cav_0.2.FEM", None, dict(h_dir=[1, 2, 3, 4], ux_dir=[1, 2, 3, 4], uy_dir=[1, 2, 3, 4])),
    12: ("ref_cdisk.1_mesh.FEM.gz", None, dict(h_dir=[1], ux_dir=[1], uy_dir=[1], tfinal=8.0)),
}


def reference_case(tt, precision=0):
    from swe import mesh as M, refcases as R
    src, jit, kw = REF_CASES[tt]
    if src == "jitter":
        nx, ny, x0, x1, y0, y1, seed = jit
        mesh = M.jittered_mesh(nx, ny, x0, x1, y0, y1, jitter=0.3, seed=seed)
    else:
        mesh = M.load_mesh_free_format(GOLDEN / src)
    return R.reference_case(tt, mesh, precision=precision, **kw)


@pytest.fixture(scope="session")
def ref_case():
    return reference_case


class OraclePerCall:
    """The per-call time loop's operators (compute_dt, set_dt, euler) over
    the oracle."""

    def __init__(self, o):
        self.o = o

    def compute_dt(self, un):
        return self.o.compute_dij(un)[1]

    def set_dt(self, dt):
        p = self.o.get_params()
        p.dt = dt
        self.o.set_params(p)

    def euler(self, un):
        return self.o.euler(un)
