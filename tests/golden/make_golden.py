"""Generate the golden fixtures in this folder by running the reference
topoptlab (stefanhiemer/topoptlab) on CPU in this container.

The reference is pure Python; it imports a few optional packages at module
level (matplotlib, cvxopt, pyamg, mmapy, meshio) that are not needed on the
paths used here (scipy-direct solve, OC optimiser, no display, no export), so
they are replaced by inert stub modules before the import.

Run:  python tests/golden/make_golden.py /path/to/reference [generator ...]
      (or set TOPOPTLAB_REFERENCE to the reference checkout and pass no path)

Outputs (small .npz files, committed):
  elements.npz     edofMat (2-D / 3-D, several nnode_dof), KE matrices,
                   create_coarse_inds arrays (the GMG index pins)
  filters.npz      matrix filter H (dense) and Hs for small 2-D / 3-D grids
  mbb2d_60x20.npz  MBB beam 60x20, ft=1, OC: obj/vol/change per iteration,
                   xPhys/u/dc/x snapshots at selected iterations, final x
  heat2d_40x40.npz heat plate 40x40, ft=0, OC (Poisson KE)
  mbb2d_60x20_ft0.npz  MBB beam 60x20 with the sensitivity filter
  cant3d_12x6x6.npz    3-D cantilever (reference callable), ft=1, 12 iterations
  cant3d_16x8x8.npz, cant3d_32x16x16.npz, cant3d_48x24x24.npz
                       the 3-D cantilever ladder (20 / 10 / 2 iterations): the
                       grids on which the multigrid hierarchy is deep; also the
                       reference's seconds per design iteration on this host
  mbb2d_60x20.log  the reference's log file of the MBB 60x20 run (verbosity 20)
  vtk.npz          what the reference's export_vtk hands to meshio (points,
                   cells, point and cell data) for a 2-D and a 3-D grid, seeded
                   fields, and what export_stl hands it for the 2-D grid,
                   recorded through a stand-in for meshio.Mesh
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if len(sys.argv) > 1:
    REF = sys.argv[1]
elif os.environ.get("TOPOPTLAB_REFERENCE"):
    REF = os.environ["TOPOPTLAB_REFERENCE"]
else:
    sys.exit("usage: make_golden.py /path/to/reference [generator ...] "
             "(or set TOPOPTLAB_REFERENCE)")


class _Inert:
    def __getattr__(self, k):
        return _Inert()

    def __call__(self, *a, **k):
        return _Inert()


def _install_stubs():
    attrs = {
        "matplotlib": [], "matplotlib.pyplot": [], "matplotlib.colors": ["Normalize"],
        "cvxopt": ["matrix", "spmatrix"], "cvxopt.cholmod": ["solve", "symbolic", "numeric"],
        "pyamg": [], "pyamg.aggregation": ["adaptive_sa_solver", "rootnode_solver",
                                            "smoothed_aggregation_solver", "pairwise_solver"],
        "pyamg.classical": ["air_solver", "ruge_stuben_solver"],
        "mmapy": ["mmasub", "gcmmasub", "asymp", "concheck", "raaupdate", "kktcheck"],
        "meshio": ["Mesh", "write", "read"],
    }
    for name, names in attrs.items():
        m = types.ModuleType(name)
        m.__path__ = []
        for a in names:
            setattr(m, a, _Inert())
        sys.modules[name] = m
    sys.modules["matplotlib"].pyplot = sys.modules["matplotlib.pyplot"]


_install_stubs()
sys.path.insert(0, REF)

import topoptlab.topology_optimization as T  # noqa: E402
from topoptlab.elements.bilinear_quadrilateral import create_edofMat as edof2d  # noqa: E402
from topoptlab.elements.trilinear_hexahedron import create_edofMat as edof3d  # noqa: E402
from topoptlab.elements.linear_elasticity_2d import lk_linear_elast_2d  # noqa: E402
from topoptlab.elements.linear_elasticity_3d import lk_linear_elast_3d  # noqa: E402
from topoptlab.elements.poisson_2d import lk_poisson_2d  # noqa: E402
from topoptlab.elements.poisson_3d import lk_poisson_3d  # noqa: E402
from topoptlab.filter.matrix_filter import assemble_matrix_filter  # noqa: E402
from topoptlab.gmg import create_coarse_inds  # noqa: E402
from topoptlab.example_bc.lin_elast import mbb_2d, cantilever_3d  # noqa: E402
from topoptlab.example_bc.heat_conduction import heatplate_2d  # noqa: E402
from topoptlab.objectives import compliance  # noqa: E402
from topoptlab.optimizer.optimality_criterion import oc_top88  # noqa: E402
import topoptlab.output_designs as OD  # noqa: E402
from topoptlab.elements.screenedpoisson_2d import lk_screened_poisson_2d  # noqa: E402
from topoptlab.elements.screenedpoisson_3d import lk_screened_poisson_3d  # noqa: E402
from topoptlab.filter.helmholtz_filter import assemble_helmholtz_filter  # noqa: E402
from topoptlab.geometries import sphere, ellipse, ball, ellipsoid  # noqa: E402
from topoptlab.example_bc.lin_elast import (cantilever_2d, cantilever_2d_wrong,  # noqa: E402
                                             cantilever_2d_twoloads_wrong)
from scipy.sparse.linalg import factorized  # noqa: E402

OUT_KW = {"file": None, "display": False, "export": False, "write_log": False,
          "profile": False, "debug": 0}


def gen_elements():
    d = {}
    for (nx, ny, nd) in [(5, 3, 1), (5, 3, 2), (60, 20, 2)]:
        d[f"edof2d_{nx}x{ny}_{nd}"] = edof2d(nelx=nx, nely=ny, nnode_dof=nd)[0]
    for (nx, ny, nz, nd) in [(4, 3, 2, 1), (4, 3, 2, 3), (6, 4, 4, 3)]:
        d[f"edof3d_{nx}x{ny}x{nz}_{nd}"] = edof3d(nelx=nx, nely=ny, nelz=nz, nnode_dof=nd)[0]
    d["KE_elast2d"] = lk_linear_elast_2d(l=np.array([1., 1.]))
    d["KE_elast3d"] = lk_linear_elast_3d(l=np.array([1., 1., 1.]))
    d["KE_poisson2d"] = lk_poisson_2d(l=np.array([1., 1.]))
    d["KE_poisson3d"] = lk_poisson_3d(l=np.array([1., 1., 1.]))
    d["KE_elast2d_rect"] = lk_linear_elast_2d(l=np.array([2., 1.]))
    d["KE_elast3d_rect"] = lk_linear_elast_3d(l=np.array([1., 2., 0.5]))
    # GMG coarse index pins (the cases of the reference's tests/test_gmg.py)
    cases = [(4, 6, None, 1, 2), (4, 6, None, 2, 2), (4, 6, 8, 1, 2), (4, 6, 8, 3, 2),
             (8, 4, 4, 3, 2), (16, 8, 8, 3, 2)]
    for (nx, ny, nz, nd, st) in cases:
        d[f"coarse_{nx}_{ny}_{nz}_{nd}_{st}"] = create_coarse_inds(
            nelx=nx, nely=ny, nelz=nz, ndof=nd, stride=st)
    # boundary-condition callables (fixed DOFs and load vectors)
    for (nx, ny) in [(60, 20), (10, 4)]:
        u, f, fixed, free, _ = mbb_2d(nelx=nx, nely=ny, ndof=2 * (nx + 1) * (ny + 1))
        d[f"bc_mbb2d_{nx}x{ny}_fixed"], d[f"bc_mbb2d_{nx}x{ny}_f"] = fixed, f[:, 0]
    for (nx, ny, nz) in [(12, 6, 6), (16, 8, 8)]:
        u, f, fixed, free, _ = cantilever_3d(nelx=nx, nely=ny, nelz=nz,
                                             ndof=3 * (nx + 1) * (ny + 1) * (nz + 1))
        d[f"bc_cant3d_{nx}x{ny}x{nz}_fixed"], d[f"bc_cant3d_{nx}x{ny}x{nz}_f"] = fixed, f[:, 0]
    for n in [40, 64, 100]:
        u, f, fixed, free, _ = heatplate_2d(nelx=n, nely=n, ndof=(n + 1) ** 2)
        d[f"bc_heat2d_{n}_fixed"], d[f"bc_heat2d_{n}_f"] = fixed, f[:, 0]
    np.savez_compressed(os.path.join(HERE, "elements.npz"), **d)


def gen_filters():
    d = {}
    for (nx, ny, nz, rmin) in [(7, 5, None, 2.4), (9, 6, None, 1.5), (6, 5, 4, 1.5),
                               (5, 4, 3, 2.4)]:
        H, Hs = assemble_matrix_filter(nelx=nx, nely=ny, nelz=nz, rmin=rmin,
                                       ndim=2 if nz is None else 3)
        key = f"{nx}_{ny}_{nz}_{rmin}"
        d["H_" + key] = H.toarray()
        d["Hs_" + key] = np.asarray(Hs).ravel()
    np.savez_compressed(os.path.join(HERE, "filters.npz"), **d)


def run_traced(name, snap_its, **kw):
    """Run the reference main() and record per-iteration state.

    compliance() sees (xPhys, u) of each iteration, oc_top88 sees
    (x, dc, dv, g) after the sensitivity filter and returns (xnew, g)."""
    rec = {"obj": [], "g": [], "xPhys": {}, "u": {}, "dc": {}, "dv": {}, "x_in": {},
           "x_out": {}, "g_in": {}}
    it = {"k": 0}

    def comp(**a):
        obj, rhs_adj, sa = compliance(**a)
        k = it["k"]
        rec["obj"].append(obj)
        if k in snap_its:
            rec["xPhys"][k] = a["xPhys"][:, 0].copy()
            rec["u"][k] = a["u"][:, 0].copy()
        return obj, rhs_adj, sa

    def oc(x, volfrac, dc, dv, g, el_flags, **k2):
        k = it["k"]
        xnew, gt = oc_top88(x=x, volfrac=volfrac, dc=dc, dv=dv, g=g, el_flags=el_flags, **k2)
        if k in snap_its:
            rec["dc"][k] = dc.copy()
            rec["dv"][k] = dv.copy()
            rec["x_in"][k] = x.copy()
            rec["x_out"][k] = xnew.copy()
            rec["g_in"][k] = g
        rec["g"].append(gt)
        it["k"] += 1
        return xnew, gt

    orig_oc = T.oc_top88
    T.oc_top88 = oc
    try:
        x, obj = T.main(obj_func=comp, optimizer="oc", output_kw=OUT_KW, **kw)
    finally:
        T.oc_top88 = orig_oc
    out = {"final_x": x[:, 0], "final_obj": np.array(obj), "g": np.array(rec["g"]),
           "obj": np.array(rec["obj"]),
           "n_iter": np.array(it["k"])}
    for key in ["xPhys", "u", "dc", "dv", "x_in", "x_out", "g_in"]:
        for k, v in rec[key].items():
            out[f"{key}_{k}"] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, name), **out)
    return x, obj, it["k"]


class _MeshRecorder:
    """Stand-in for meshio.Mesh: keeps what export_vtk passes to it."""
    last = None

    def __init__(self, points, cells, point_data=None, cell_data=None):
        _MeshRecorder.last = dict(points=np.asarray(points), cells=cells,
                                  point_data=point_data or {}, cell_data=cell_data or {})

    def write(self, filename):
        _MeshRecorder.last["filename"] = filename


def gen_vtk():
    OD.Mesh = _MeshRecorder
    rng = np.random.default_rng(7)
    d = {}
    for tag, (nx, ny, nz, nd) in {"2d": (4, 3, None, 2), "3d": (3, 2, 2, 3)}.items():
        nel = nx * ny * (nz or 1)
        nnodes = (nx + 1) * (ny + 1) * ((nz or 0) + 1)
        xPhys = rng.uniform(0, 1, (nel, 1))
        x = rng.uniform(0, 1, (nel, 1))
        u = rng.standard_normal((nnodes * nd, 2))
        f = rng.standard_normal((nnodes * nd, 2))
        OD.export_vtk(filename="out", nelx=nx, nely=ny, nelz=nz, xPhys=xPhys, x=x, u=u, f=f,
                      volfrac=0.4)
        m = _MeshRecorder.last
        d[f"{tag}_points"] = m["points"]
        d[f"{tag}_cells"] = np.asarray(m["cells"][0][1])
        d[f"{tag}_celltype"] = np.array(m["cells"][0][0])
        for k, v in m["point_data"].items():
            d[f"{tag}_pd_{k}"] = np.asarray(v)
        for k, v in m["cell_data"].items():
            d[f"{tag}_cd_{k}"] = np.asarray(v[0])
        d[f"{tag}_in_xPhys"], d[f"{tag}_in_x"], d[f"{tag}_in_u"], d[f"{tag}_in_f"] = xPhys, x, u, f
        if nz is None:      # export_stl is 2-D (output_designs.py:181-230)
            # As written it indexes the (nel, 4) cell array with threshold()'s
            # (nel, 1) mask, which NumPy rejects; recorded with the mask
            # flattened, its evident intent.
            orig = OD.threshold
            OD.threshold = lambda xp, vf: orig(xp, vf)[:, 0]
            try:
                OD.export_stl(filename="out", nelx=nx, nely=ny, xPhys=xPhys, volfrac=0.4)
            finally:
                OD.threshold = orig
            m = _MeshRecorder.last
            d["stl_points"] = m["points"]
            d["stl_celltype"] = np.array(m["cells"][0][0])
            d["stl_tris"] = np.asarray(m["cells"][0][1])
    np.savez_compressed(os.path.join(HERE, "vtk.npz"), **d)


def gen_helmholtz():
    """Screened Poisson element matrices, the Helmholtz filter applied to seeded
    fields (filter/helmholtz_filter.py), and the reference design loop with
    filter_mode="helmholtz" on the 60x20 MBB beam (tests/test_compliance.py:11-12)."""
    rng = np.random.default_rng(11)
    d = {}
    for rmin in (2.4, 1.5):
        k = (rmin / (2 * np.sqrt(3))) ** 2
        d[f"KF2d_{rmin}"] = lk_screened_poisson_2d(k=k, l=np.array([1., 1.]))
        d[f"KF3d_{rmin}"] = lk_screened_poisson_3d(k=k, l=np.array([1., 1., 1.]))
    d["KF2d_rect"] = lk_screened_poisson_2d(k=0.3, l=np.array([2., 0.5]))
    for (nx, ny, rmin) in [(7, 5, 2.4), (12, 8, 1.5)]:
        # the operators main() uses (topology_optimization.py:360-365, 569, 647);
        # the HelmholtzFilter class itself is abstract (no vol_conserv)
        KF, TF = assemble_helmholtz_filter(nelx=nx, nely=ny, rmin=rmin)
        lu_solve = factorized(KF)
        x = rng.uniform(0.0, 1.0, (nx * ny, 1))
        dx = rng.standard_normal((nx * ny, 1))
        key = f"{nx}_{ny}_{rmin}"
        d["x_" + key], d["dx_" + key] = x[:, 0], dx[:, 0]
        d["y_" + key] = (TF.T @ lu_solve(TF @ x))[:, 0]
        d["dy_" + key] = (TF.T @ lu_solve(TF @ (dx * x)) / np.maximum(0.001, x))[:, 0]
    np.savez_compressed(os.path.join(HERE, "helmholtz.npz"), **d)
    for ft in (1, 0):
        r = run_traced(f"mbb2d_60x20_helmholtz_ft{ft}.npz", {0, 1, 2},
                       nelx=60, nely=20, volfrac=0.5, rmin=2.4, ft=ft, bcs=mbb_2d,
                       filter_mode="helmholtz")
        print(f"mbb helmholtz ft{ft}", r[1], r[2])


def gen_passive():
    """tests/test_passive.py:8-34 of the reference: the 60x20 cantilever with
    a passive disc from geometries.sphere, ft=0, OC (golden 221.9720563724),
    plus the flags of sphere and ellipse for a few shapes."""
    d = {}
    for (nx, ny, c, r) in [(60, 20, (60 / 3 - 1, 20 / 2 - 1), 20 / 3), (9, 7, (4.0, 3.0), 2.5)]:
        d[f"sphere_{nx}_{ny}"] = sphere(nelx=nx, nely=ny, center=c, radius=r)
    d["ellipse_12_8"] = ellipse(nelx=12, nely=8, center=(5.0, 3.5), ax_half_lengths=(4.0, 2.0),
                                fill_value=2)
    d["ball_8_6_5"] = ball(nelx=8, nely=6, nelz=5, center=(3.5, 2.0, 2.5), radius=2.2)
    d["ellipsoid_8_6_5"] = ellipsoid(nelx=8, nely=6, nelz=5, center=(3.0, 2.5, 2.0),
                                     ax_half_lengths=(3.0, 1.5), fill_value=2)
    for name, fn in (("wrong", cantilever_2d_wrong), ("twoloads_wrong", cantilever_2d_twoloads_wrong)):
        u, f, fixed, free, _ = fn(nelx=12, nely=5, ndof=2 * 13 * 6)
        d[f"bc_cant2d_{name}_fixed"], d[f"bc_cant2d_{name}_f"] = fixed, f
    np.savez_compressed(os.path.join(HERE, "geometries.npz"), **d)
    flags = sphere(nelx=60, nely=20, center=(60 / 3 - 1, 20 / 2 - 1), radius=20 / 3)
    r = run_traced("cant2d_60x20_passive.npz", {0, 1},
                   nelx=60, nely=20, volfrac=0.5, rmin=2.4, ft=0, bcs=cantilever_2d,
                   el_flags=flags, filter_mode="matrix")
    print("cant2d passive", r[1], r[2])


def gen_slow_cantilevers():
    """The reference's slow compliance cases (tests/test_compliance.py:38-59):
    cantilever_2d_wrong 160x100 (61.4282510690) and
    cantilever_2d_twoloads_wrong 150x150 (69.2037375459), ft=0, rmin 6."""
    r = run_traced("cant2d_wrong_160x100.npz", {0},
                   nelx=160, nely=100, volfrac=0.4, rmin=6.0, ft=0, bcs=cantilever_2d_wrong,
                   filter_mode="matrix")
    print("cant2d wrong", r[1], r[2])
    r = run_traced("cant2d_twoloads_wrong_150x150.npz", {0},
                   nelx=150, nely=150, volfrac=0.4, rmin=6.0, ft=0,
                   bcs=cantilever_2d_twoloads_wrong, filter_mode="matrix")
    print("cant2d twoloads wrong", r[1], r[2])
    for name in ("cant2d_wrong_160x100.npz", "cant2d_twoloads_wrong_150x150.npz"):
        path = os.path.join(HERE, name)
        d = dict(np.load(path))
        np.savez_compressed(path, **{k: d[k] for k in ("obj", "g", "final_obj", "final_x",
                                                        "n_iter")})


def gen_convolution():
    """The reference's convolution-mode filter (filter/convolution_filter.py
    with scipy.ndimage.convolve, as tests/test_filters.py runs it) on seeded
    fields: the outputs the matrix filter must reproduce."""
    from functools import partial
    from scipy.ndimage import convolve
    from topoptlab.filter.convolution_filter import assemble_convolution_filter
    from topoptlab.utils import map_eltoimg, map_imgtoel, map_eltovoxel, map_voxeltoel
    rng = np.random.default_rng(2)
    d = {}
    for (nx, ny, nz, rmin) in [(10, 10, None, 2.4), (20, 10, None, 2.4), (10, 20, None, 2.4),
                               (10, 10, 10, 2.4), (20, 10, 10, 2.4), (10, 20, 10, 2.4),
                               (9, 6, 5, 1.5)]:
        ndim = 2 if nz is None else 3
        if ndim == 2:
            mp, imp = partial(map_eltoimg, nelx=nx, nely=ny), partial(map_imgtoel, nelx=nx, nely=ny)
        else:
            mp = partial(map_eltovoxel, nelx=nx, nely=ny, nelz=nz)
            imp = partial(map_voxeltoel, nelx=nx, nely=ny, nelz=nz)
        h, hs = assemble_convolution_filter(nelx=nx, nely=ny, nelz=nz, rmin=rmin, mapping=mp,
                                            invmapping=imp)
        n = nx * ny * (nz or 1)
        x = rng.uniform(0.0, 1.0, (n, 1))
        y = imp(convolve(mp(x), h, mode="constant", axes=(0, 1, 2)[:ndim], cval=0)) / hs
        key = f"{nx}_{ny}_{nz}_{rmin}"
        d["x_" + key], d["y_" + key] = x[:, 0], np.asarray(y).reshape(-1)
    np.savez_compressed(os.path.join(HERE, "convolution.npz"), **d)


def gen_stiffness():
    """The reference's recorded SIMP systems (examples/linsolvers:
    K[free][:, free] of design iteration 25 and its xPhys, MBB 60x20 and heat
    plate 40x40): the densities, the matrix diagonal and its product with a
    seeded vector, enough to pin an assembly of K from the densities."""
    import scipy.sparse as sp
    base = os.path.join(REF, "examples", "linsolvers")
    rng = np.random.default_rng(4)
    d = {}
    for tag in ("mbb2d_60x20-2.4-0.5-0_25", "heatplate2d_40x40-1.2-0.4-0_25"):
        K = sp.load_npz(os.path.join(base, f"stiffness-matrix_{tag}.npz")).tocsr()
        x = np.loadtxt(os.path.join(base, f"xPhys_{tag}.csv"), delimiter=",").reshape(-1)
        v = rng.standard_normal(K.shape[0])
        key = tag.split("-")[0]
        d[key + "_xPhys"], d[key + "_v"] = x, v
        d[key + "_Kv"], d[key + "_diag"] = K @ v, K.diagonal()
    np.savez_compressed(os.path.join(HERE, "stiffness.npz"), **d)


def gen_ladder():
    """The 3-D cantilever (reference cantilever_3d callable, volfrac 0.3,
    rmin 1.5, ft=1, OC, scipy-direct) on the grids 16x8x8 (20 iterations),
    32x16x16 (10) and 48x24x24 (2): compliance per iteration, the final
    design, the last iteration's xPhys and filtered dc (up to 32x16x16) and
    u (16x8x8), plus the reference's wall time per design iteration."""
    import time
    for (nx, ny, nz, nit) in [(16, 8, 8, 20), (32, 16, 16, 10), (48, 24, 24, 2)]:
        name = f"cant3d_{nx}x{ny}x{nz}.npz"
        t0 = time.perf_counter()
        r = run_traced(name, {nit - 1}, nelx=nx, nely=ny, nelz=nz, volfrac=0.3, rmin=1.5,
                       ft=1, bcs=cantilever_3d, nouteriter=nit)
        sec = (time.perf_counter() - t0) / nit
        path = os.path.join(HERE, name)
        d = dict(np.load(path))
        keep = {k: d[k] for k in ("obj", "g", "final_x", "final_obj", "n_iter")}
        last = nit - 1
        # the last iteration's fields where they keep the fixture small
        if nx <= 32:
            keep["xPhys_last"] = d[f"xPhys_{last}"]
            keep["dc_last"] = d[f"dc_{last}"]
        if nx <= 16:
            keep["u_last"] = d[f"u_{last}"]
        keep["seconds_per_iteration"] = np.array(sec)
        np.savez_compressed(path, **keep)
        print("ladder", nx, ny, nz, r[1], f"{sec:.2f} s/iteration")


def gen_log():
    """The reference's log file (SimpleLogger, verbosity 20) of the MBB beam
    60x20 run with the density filter (tests/test_compliance.py:10 set-up)."""
    import tempfile
    with tempfile.TemporaryDirectory() as tmp:
        base = os.path.join(tmp, "mbb")
        kw = dict(OUT_KW, write_log=True, file=base, verbosity=20)
        T.main(nelx=60, nely=20, volfrac=0.5, rmin=2.4, ft=1, bcs=mbb_2d, optimizer="oc",
               lin_solver_kw={"name": "scipy-direct"}, output_kw=kw)
        text = open(base + ".log").read()
    with open(os.path.join(HERE, "mbb2d_60x20.log"), "w") as f:
        f.write(text)
    print("log lines", len(text.splitlines()))


GENERATORS = {"log": lambda: gen_log(), "ladder": lambda: gen_ladder(), "vtk": lambda: gen_vtk(),
              "helmholtz": lambda: gen_helmholtz(), "stiffness": lambda: gen_stiffness(),
              "convolution": lambda: gen_convolution(),
              "passive": lambda: gen_passive(), "slow": lambda: gen_slow_cantilevers()}


def main():
    # optional names after the reference path regenerate only those fixtures
    if len(sys.argv) > 2:
        for name in sys.argv[2:]:
            GENERATORS[name]()
        return
    gen_vtk()
    gen_helmholtz()
    gen_passive()
    gen_convolution()
    gen_stiffness()
    gen_elements()
    gen_filters()
    r = run_traced("mbb2d_60x20.npz", {0, 1, 2, 24, 143},
                   nelx=60, nely=20, volfrac=0.5, rmin=2.4, ft=1, bcs=mbb_2d)
    print("mbb ft1", r[1], r[2])
    r = run_traced("mbb2d_60x20_ft0.npz", {0, 1, 2},
                   nelx=60, nely=20, volfrac=0.5, rmin=2.4, ft=0, bcs=mbb_2d)
    print("mbb ft0", r[1], r[2])
    r = run_traced("heat2d_40x40.npz", {0, 1, 2},
                   nelx=40, nely=40, volfrac=0.4, rmin=1.2, ft=0, bcs=heatplate_2d,
                   lk=lk_poisson_2d)
    print("heat", r[1], r[2])
    r = run_traced("cant3d_12x6x6.npz", {0, 1, 11},
                   nelx=12, nely=6, nelz=6, volfrac=0.3, rmin=1.5, ft=1,
                   bcs=cantilever_3d, nouteriter=12)
    print("cant3d", r[1], r[2])
    gen_ladder()
    gen_log()


if __name__ == "__main__":
    main()
