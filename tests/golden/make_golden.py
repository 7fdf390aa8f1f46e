"""Generate the committed golden fixtures of tests/golden/.

Run where a checkout of the reference exists (read-only is enough), giving
its root directory:   python tests/golden/make_golden.py REFERENCE_ROOT

Fixtures written (all small, numpy .npz):
  mesh_cav_{0.2,0.1,0.05}.npz  MESHES/PARABOLOID/cav_*.FEM read and renumbered
                               like prep_mesh.f90 (jj, rr, jjs, sides).
  pin_backup_cav02.npz         SOURCES/BACKUP/hinit.plt and bath.plt: the
                               reference's own dump of node coordinates, h0 and
                               bathymetry per node (type_test 5 on cav_0.2,
                               written by an older revision without +htiny).
  pin_lis.npz                  it_max and relative L1 errors recorded in
                               PARABOLOID/lis_{h}_type2_lim (older revision).
  ref_{bath,h_1,hpz_1}.vtk.gz  SOURCES/BACKUP/*.vtk, the reference's own vtk_2d
                               output on cav_0.2 (gzip of the files as shipped):
                               pins the VTK text byte for byte.
  ref_cav_0.2.FEM              MESHES/PARABOLOID/cav_0.2.FEM as shipped: the
                               .FEM reader's input for the mesh fixture test.
  ref_{rectangle.1,cdisk.1_mesh,dam_cav_0.25,bump_cav_0.3}.FEM.gz
                               MESHES/SGN_CANAL/rectangle.1.FEM,
                               PARABOLOID/cdisk.1_mesh.FEM, DAM_BREAK/cav_0.25.FEM,
                               BUMP_3_1/cav_0.3.FEM (gzip of the files as
                               shipped): the meshes of the reference's test
                               cases 13, 12, 4 and 2/3/6/7.
  ref_data_{sources,paraboloid,backup}.txt
                               SOURCES/data, PARABOLOID/data, SOURCES/BACKUP/data
                               as shipped: inputs for the data-file reader.
  oracle_*.npz                 FP64 oracle trajectories (regression vectors
                               for the oracle itself and GPU parity vectors).
"""
from __future__ import annotations

import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
REF = Path(sys.argv[1]) if len(sys.argv) > 1 else None
sys.path.insert(0, str(REPO / "shallow-water-eric_gb300"))
sys.path.insert(0, str(REPO))

from swe import mesh as M, cases as C  # noqa: E402
import oracle  # noqa: E402


def parse_plt(path):
    """(node -> (x, y, value)) from a PLTMTV CONTCURVE dump (sub_plot.f90:703-778)."""
    nodes = {}
    for line in Path(path).read_text().splitlines():
        parts = line.split()
        if len(parts) != 4 or line.startswith(("$", "%")):
            continue
        x, y, v, n = float(parts[0]), float(parts[1]), float(parts[2]), int(parts[3])
        nodes[n] = (x, y, v)
    idx = np.array(sorted(nodes))
    arr = np.array([nodes[i] for i in idx])
    return idx, arr


def main():
    if REF is None or not (REF / "SOURCES" / "update.f90").exists():
        sys.exit("usage: python tests/golden/make_golden.py REFERENCE_ROOT (the reference checkout's root)")
    for h in ("0.2", "0.1", "0.05"):
        m = M.load_mesh_free_format(REF / "MESHES/PARABOLOID" / f"cav_{h}.FEM")
        np.savez_compressed(HERE / f"mesh_cav_{h}.npz", jj=m["jj"], rr=m["rr"], jjs=m["jjs"], sides=m["sides"])
    idx, hinit = parse_plt(REF / "SOURCES/BACKUP/hinit.plt")
    idx2, bath = parse_plt(REF / "SOURCES/BACKUP/bath.plt")
    assert np.array_equal(idx, idx2)
    np.savez_compressed(HERE / "pin_backup_cav02.npz", node=idx, x=hinit[:, 0], y=hinit[:, 1], h0=hinit[:, 2],
                        bath=bath[:, 2])
    it_max, l1 = [], []
    for h in ("0.2", "0.1", "0.05", "0.025", "0.0125"):
        txt = (REF / "PARABOLOID" / f"lis_{h}_type2_lim").read_text().splitlines()
        it_max.append(int(txt[2].split()[-1]))
        l1.append(float(re.findall(r"[-+0-9.E]+", txt[3])[-1]))
    np.savez(HERE / "pin_lis.npz", h=np.array([0.2, 0.1, 0.05, 0.025, 0.0125]), it_max=np.array(it_max),
             l1=np.array(l1), cfl=0.3)

    (HERE / "ref_cav_0.2.FEM").write_bytes((REF / "MESHES/PARABOLOID/cav_0.2.FEM").read_bytes())
    for tag, rel in (("sources", "SOURCES/data"), ("paraboloid", "PARABOLOID/data"),
                     ("backup", "SOURCES/BACKUP/data")):
        (HERE / f"ref_data_{tag}.txt").write_bytes((REF / rel).read_bytes())
    import gzip
    for name in ("bath", "h_1", "hpz_1"):
        data = (REF / "SOURCES/BACKUP" / f"{name}.vtk").read_bytes()
        with gzip.GzipFile(HERE / f"ref_{name}.vtk.gz", "wb", mtime=0) as f:
            f.write(data)

    for name, rel in (("rectangle.1", "SGN_CANAL/rectangle.1.FEM"), ("cdisk.1_mesh", "PARABOLOID/cdisk.1_mesh.FEM"),
                      ("dam_cav_0.25", "DAM_BREAK/cav_0.25.FEM"), ("bump_cav_0.3", "BUMP_3_1/cav_0.3.FEM")):
        with gzip.GzipFile(HERE / f"ref_{name}.FEM.gz", "wb", mtime=0) as f:
            f.write((REF / "MESHES" / rel).read_bytes())

    # oracle trajectories
    m = dict(np.load(HERE / "mesh_cav_0.2.npz"))
    case = C.thacker_case(m, periods=1.0, cfl=0.3)
    o = oracle.Oracle(m["jj"], m["rr"])
    o.set_params(oracle.Params(*case.params.fields()))
    o.set_bath(case.bath)
    for comp, js, vals in case.dirichlet:
        o.set_dirichlet(comp, js, vals)
    u = case.u0.copy(order="F")
    states, times = [u.copy()], [0.0]
    t = 0.0
    for s in range(40):
        t = o.rk3_step(u, t)
        if (s + 1) % 10 == 0:
            states.append(u.copy()); times.append(t)
    np.savez_compressed(HERE / "oracle_thacker_cav02.npz", states=np.array(states), times=np.array(times),
                        steps_per_state=10)

    case = C.dam_break_case(n=21, tfinal=0.05)
    mm = case.mesh
    o = oracle.Oracle(mm["jj"], mm["rr"])
    o.set_params(oracle.Params(*case.params.fields()))
    o.set_bath(case.bath)
    for comp, js, vals in case.dirichlet:
        o.set_dirichlet(comp, js, vals)
    u = case.u0.copy(order="F")
    t, n = o.run(u, 0.0, case.tfinal)
    np.savez_compressed(HERE / "oracle_dam21.npz", u=u, time=t, nsteps=n)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
