"""Drop-in ``main`` for the reference driver topoptlab.topology_optimization.main
(topology_optimization.py:47-688), running every design iteration on the GPU.

Same signature, same return value ``(x, obj)`` (x of shape (nel, 1), obj the
compliance of the last solved design), same per-iteration log line
``it.: {k} obj.: {obj:.10f} vol.: {vol:.10f} ch.: {change:.10f}``
(:669-670) and the same stopping rule ``change < 0.01`` (:672).

Supported: quad4 / hex8 structured grids, ``lk`` callables returning the
element matrix (elasticity or Poisson), ``bcs`` callables of the reference
example_bc signature (any number of load cases, no springs), ``ft`` in {-1, 0, 1}
with ``filter_mode`` "matrix" or "convolution" (identical operators), or
"helmholtz" (the PDE filter, ft in {0, 1}, 2-D like the reference's
filter/helmholtz_filter.py:177-180),
``optimizer="oc"``, SIMP (``matinterpol_kw`` eps / penal), ``el_flags``.
Anything else raises ValueError, as the reference does for unknown options
(:262, :367).  There is no CPU path.

Solver selection (``lin_solver_kw["name"]``):
  "gb300-gmgpcg" (default)  GMG-preconditioned CG to ``rtol`` (default 1e-8)
  "gb300-pcg"               CG preconditioned by ``preconditioner_kw["name"]``
  any reference solver name ("scipy-direct", "scipy-cg", "cvxopt-cholmod",
  "topoptlab-pcg", ...) runs the same GPU GMG-PCG; the direct-solver names
  use rtol 1e-12 so the result matches a direct solve.
``preconditioner_kw``: name "gb300-gmg" (default) or "gb300-jacobi";
``nlevels`` (0 = automatic), ``nsmooth`` (2), ``omega`` (0.6),
``precision`` ("fp64" or "mixed"), ``inner_rtol`` (1e-4), ``learned`` (False).
``learned`` carries a trained network (no counterpart in the reference): the
flat parameter vector of a ``learned.LearnedWarmStart`` (its ``params()``), or
the path of a ``.npy`` file holding it, optionally as
``{"params": ..., "mode": "warm_start" | "coarse_correction" | "both"}``
(default "warm_start").  The network then gives each solve its warm start
(and with "coarse_correction" the FP32 PCG its deflation vector); it needs a
3-D elasticity problem with ``precision="mixed"`` and multigrid.
``learned=True`` without parameters raises ValueError, like the reference's
unknown-option errors.
"""
from __future__ import annotations

import warnings
from cProfile import Profile
from typing import Callable, Dict, List, Tuple, Union

import numpy as np

from . import _lib
from .context import GpuProblem
from .elements import lk_linear_elast_2d, lk_linear_elast_3d
from .example_bc import mbb_2d
from .log_utils import EmptyLogger, SimpleLogger
from .material_interpolation import simp, simp_dx
from .objectives import compliance
from .output_designs import export_vtk
from .utils import default_outputkw, check_output_kw, check_simulation_params

_DIRECT = {"scipy-direct", "scipy-lu", "cvxopt-cholmod"}
_ITERATIVE = {"scipy-cg", "scipy-bicg", "scipy-cgs", "scipy-gmres", "scipy-lgmres",
              "scipy-minres", "scipy-qmr", "scipy-tfqmr", "scipy-gcrotmk", "topoptlab-pcg",
              "topoptlab-cg"}


def solver_options(lin_solver_kw: Dict, preconditioner_kw: Dict) -> Dict:
    """Translate the reference's solver / preconditioner dicts to GPU options."""
    name = lin_solver_kw.get("name", "gb300-gmgpcg")
    pname = preconditioner_kw.get("name", None)
    opts = dict(precond="gb300-gmg", precision="fp64", nlevels=0, nsmooth=2, omega=0.6,
                rtol=1e-8, maxiter=2000, inner_rtol=1e-4, learned=False, unsmoothed=0,
                nsmooth_coarse=0)
    if name in _DIRECT:
        opts["rtol"] = 1e-12
    elif name in ("gb300-gmgpcg", "gb300-pcg") or name in _ITERATIVE:
        pass
    else:
        raise ValueError("Unknown solver: ", name)
    if "rtol" in lin_solver_kw:
        opts["rtol"] = float(lin_solver_kw["rtol"])
    if "maxiter" in lin_solver_kw:
        opts["maxiter"] = int(lin_solver_kw["maxiter"])
    if name == "gb300-pcg" and pname in ("gb300-jacobi",):
        opts["precond"] = "gb300-jacobi"
    elif pname in ("gb300-jacobi",):
        opts["precond"] = "gb300-jacobi"
    elif pname not in (None, "gb300-gmg") and not str(pname).startswith(("pyamg-", "scipy-")):
        raise ValueError("Unknown preconditioner: ", pname)
    for key in ("nlevels", "nsmooth", "maxiter", "unsmoothed", "nsmooth_coarse"):
        if key in preconditioner_kw:
            opts[key] = int(preconditioner_kw[key])
    for key in ("omega", "inner_rtol"):
        if key in preconditioner_kw:
            opts[key] = float(preconditioner_kw[key])
    if "precision" in preconditioner_kw:
        opts["precision"] = preconditioner_kw["precision"]
    if "learned" in preconditioner_kw:
        opts["learned"] = preconditioner_kw["learned"]
    return opts


def learned_network(spec):
    """(params, mode) of preconditioner_kw["learned"]; (None, 0) for none."""
    if spec is None or spec is False:
        return None, 0
    mode = "warm_start"
    if isinstance(spec, dict):
        mode = spec.get("mode", "warm_start")
        spec = spec.get("params")
    if spec is True or spec is None:
        raise ValueError("preconditioner_kw['learned'] needs trained network parameters "
                         "(LearnedWarmStart.params() or the path of a .npy file holding them)")
    if isinstance(spec, str):
        spec = np.load(spec)
    params = np.ascontiguousarray(np.asarray(spec, dtype=np.float32).reshape(-1))
    if params.size == 0:
        raise ValueError("preconditioner_kw['learned']: empty parameter vector")
    return params, mode


def _name(fn) -> str:
    return getattr(fn, "__name__", "")


def main(nelx: int, nely: int,
         volfrac: float,
         rmin: float,
         ft: int = 1,
         filter_kw: Dict = {},
         simulation_kw: Dict = {"grid": "regular", "element order": 1, "meshfile": None},
         nelz: Union[None, int] = None,
         filter_mode: str = "matrix",
         lin_solver_kw: Dict = {"name": "gb300-gmgpcg"},
         preconditioner_kw: Dict = {"name": "gb300-gmg"},
         assembly_mode: str = "full",
         materials_kw: Dict = {"E": 1.},
         body_forces_kw: Dict = {},
         bcs: Callable = mbb_2d,
         lk: Union[None, Callable] = None,
         l: Union[float, List, np.ndarray] = 1.,
         obj_func: Callable = compliance,
         obj_kw: Dict = {},
         matinterpol: Callable = simp,
         matinterpol_dx: Callable = simp_dx,
         matinterpol_kw: Dict = {"eps": 1e-9, "penal": 3.},
         el_flags: Union[None, np.ndarray] = None,
         optimizer: str = "mma",
         optimizer_kw: Union[None, Dict] = None,
         mix: Union[None, float] = None,
         accelerator_kw: Dict = {"accel_freq": 4, "accel_start": 20, "max_history": 0,
                                 "accelerator": None},
         nouteriter: int = 2000, ninneriter: int = 15,
         output_kw: Dict = default_outputkw(),
         device: int = 0) -> Tuple[np.ndarray, float]:
    """Topology optimisation with SIMP and OC on the GPU; see the module doc."""
    check_output_kw(output_kw)
    check_simulation_params(simulation_kw)
    # host-side profile of the run, as topology_optimization.py:163-165 / 681-683
    profiler = None
    if output_kw.get("profile"):
        profiler = Profile()
        profiler.enable()
    ndim = 2 if nelz is None else 3
    # ---- options the GPU path implements (everything else: ValueError) ----
    if optimizer != "oc":
        raise ValueError("Unknown optimizer: ", optimizer,
                         "(the GPU path implements the optimality criteria method 'oc')")
    if not isinstance(ft, (int, np.integer)) or ft not in (-1, 0, 1):
        raise ValueError(f"Unknown filter. ft: {ft} filter_mode {filter_mode}")
    if filter_mode not in ("matrix", "convolution") and not (filter_mode == "helmholtz"
                                                            and ft in (0, 1)):
        raise ValueError(f"Unknown filter. ft: {ft} filter_mode {filter_mode}")
    if filter_mode == "helmholtz" and ndim == 3:
        # assemble_helmholtz_filter raises this for 3-D (filter/helmholtz_filter.py:180)
        raise NotImplementedError("3D not yet completely implemented.")
    if len(body_forces_kw) > 0:
        raise ValueError("body forces are not supported by the GPU path")
    if mix is not None or (accelerator_kw is not None and accelerator_kw.get("accelerator") is not None):
        raise ValueError("mixing / accelerators are not supported by the GPU path")
    if _name(obj_func) != "compliance":
        raise ValueError("the GPU path implements the compliance objective only")
    if _name(matinterpol) != "simp" or _name(matinterpol_dx) != "simp_dx":
        raise ValueError("the GPU path implements SIMP material interpolation only")
    if assembly_mode not in ("full", "lower"):
        raise ValueError(f"Unknown assembly_mode {assembly_mode}")
    opts = solver_options(lin_solver_kw, preconditioner_kw)
    net_params, net_mode = learned_network(opts.pop("learned"))
    if net_params is not None and (ndim != 3 or opts["precision"] != "mixed"
                                   or opts["precond"] != "gb300-gmg"):
        raise ValueError("the learned network needs a 3-D problem with precision='mixed' and "
                         "the multigrid preconditioner")
    eps = float(matinterpol_kw.get("eps", 1e-9))
    penal = float(matinterpol_kw.get("penal", 3.0))
    # ---- logging (log_utils.SimpleLogger semantics) ----
    if output_kw["write_log"]:
        log = SimpleLogger(file=output_kw["file"], verbosity=output_kw["verbosity"])
        log.info(f"optimizer {optimizer}")
        log.info(f"number of spatial dimensions: {ndim}")
        log.info("elements: " + " x ".join([f"{nelx}", f"{nely}", f"{nelz}"][:ndim]))
        log.info(f"volfrac: {volfrac} rmin: {rmin}")
        log.info("filter: " + ["Sensitivity based", "Density based", "Haeviside Guest",
                               "Haeviside complement Sigmund 2007", "Haeviside eta projection",
                               "Volume Preserving eta projection", "No filter"][ft])
        log.info(f"filter mode: {filter_mode}")
    else:
        log = EmptyLogger()
    if output_kw["display"]:
        warnings.warn("display is not available on the GPU path; continuing without it")
    # ---- problem set-up (topology_optimization.py:203-370) ----
    if isinstance(l, float):
        l = np.array([l for _ in range(ndim)])
    if lk is None:
        lk = lk_linear_elast_2d if ndim == 2 else lk_linear_elast_3d
    KE = np.asarray(lk(l=l), dtype=np.float64)
    nnode_dof = int(KE.shape[-1] / 2 ** ndim)
    ndof = nnode_dof * int(np.prod(np.array([nelx, nely, nelz][:ndim]) + 1))
    u, f, fixed, free, springs = bcs(nelx=nelx, nely=nely, nelz=nelz, ndof=ndof)
    if springs is not None:
        raise ValueError("springs are not supported by the GPU path")
    f = np.asarray(f, dtype=np.float64)
    if f.ndim == 1:
        f = f[:, None]
    # several columns = several load cases: one solve each, compliance and
    # sensitivities summed (topology_optimization.py:446-500)
    prob = GpuProblem(nelx, nely, nelz, KE, fixed, f, volfrac, rmin, ft=int(ft),
                      eps=eps, penal=penal, el_flags=el_flags, device=device,
                      filter_mode=filter_mode, filter_l=l,
                      learned=net_mode if net_params is not None else False, **opts)
    net = None
    if net_params is not None:
        from .learned import LearnedWarmStart
        try:
            net = LearnedWarmStart(prob, capacity=0)
            if net.info()["nparams"] != net_params.size:
                raise ValueError(f"preconditioner_kw['learned']: {net_params.size} parameters, "
                                 f"the network has {net.info()['nparams']}")
            net.set_params(net_params)
            net.attach(prob)
        except Exception:
            if net is not None:
                net.close()
            prob.close()
            raise
    obj = 0.0

    def export(name):
        # output_designs.export_vtk with the fields the reference exports (:663-680)
        export_vtk(filename=name, nelx=nelx, nely=nely, nelz=nelz,
                   xPhys=prob.get(_lib.TG_FIELD_XPHYS), x=prob.get(_lib.TG_FIELD_X),
                   u=prob.get(_lib.TG_FIELD_U).reshape(ndof, -1), f=f, volfrac=volfrac)

    try:
        for loop in range(nouteriter):
            it = prob.step()
            obj = it.obj
            log.perf(f"PCGit. {it.pcg_iters} rel.res. {it.rel_res:.3e} "
                     f"vcycles {it.vcycles} refinements {it.refinements}")
            if output_kw.get("output_movie"):
                export("_".join([output_kw["file"], str(loop).zfill(len(str(nouteriter)))]))
            log.info("it.: {0} obj.: {1:.10f} vol.: {2:.10f} ch.: {3:.10f}".format(
                loop + 1, obj, it.vol, it.change))
            if it.change < 0.01:
                break
        x = prob.get(_lib.TG_FIELD_X)
        if output_kw["export"]:
            export(output_kw["file"])
    finally:
        if net is not None:
            net.close()
        prob.close()
    if profiler is not None:
        profiler.disable()
        profiler.dump_stats(output_kw["file"] + ".prof")
    return x.reshape(-1, 1), obj
