"""Alignment caller of the volume path: similarity measures, the damped Newton
optimiser and the moment-matching warm start (reference cpp/app/align,
headless: similarity_measure.hpp, optimizer.hpp, warm_start.hpp).

Geometry 1 stays at the identity; geometry 2 moves under an AffineDoF
(12 DoFs [t, A row-major]).  The objective is -log(similarity).  An
``Aligner`` keeps the k-grid and both geometries resident on the device, so
each evaluation recomputes only geometry 2's form factors (and, for
derivatives, its DoF Jacobian) and one small contraction.  The free functions
mirror the reference's signatures and build a fresh aligner per call, like
the reference rebuilds its device state per call.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from .geometry import Geometry, SceneObject
from .kgrid import KGrid

SIM_OCHIAI, SIM_JACCARD, SIM_DICE = _lib.SIM_OCHIAI, _lib.SIM_JACCARD, _lib.SIM_DICE
SIM_FUNC_ONLY, SIM_GRADIENT, SIM_HESSIAN = _lib.SIM_FUNC_ONLY, _lib.SIM_GRADIENT, _lib.SIM_HESSIAN
SIM_FUNC_GRAD, SIM_ALL = _lib.SIM_FUNC_GRAD, _lib.SIM_ALL
MEASURES = {"ochiai": SIM_OCHIAI, "jaccard": SIM_JACCARD, "dice": SIM_DICE}
IDENTITY = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1], dtype=np.float64)


@dataclass
class SimilarityResult:
    """similarity_measure.hpp:27-32."""
    value: float                   # -log(similarity)
    gradient: np.ndarray | None    # of the value w.r.t. the 12 DoFs
    hessian: np.ndarray | None     # Gauss-Newton Hessian of the value
    similarity: float


@dataclass
class OptimizationState:
    """optimizer.hpp:12-19 (plus accepted steps and similarity evaluations)."""
    dofs: np.ndarray
    similarity: float
    similarity_loss: float
    iteration: int
    converged: bool
    status: str
    steps: int = 0
    evaluations: int = 0


def _geom_obj(geom: Geometry) -> _lib.PiObject:
    e = geom.elems
    return _lib.PiObject(geom.type, _lib.DOF_AFFINE, len(e), e.ctypes.data if len(e) else None, 12,
                         IDENTITY.ctypes.data)


def _measure(m) -> int:
    if isinstance(m, str):
        return MEASURES[m.lower()]
    return int(m)


def _dofs12(d) -> np.ndarray:
    d = np.ascontiguousarray(np.asarray(d, dtype=np.float64).reshape(-1))
    if d.shape != (12,):
        raise ValueError("AffineDoF vectors have 12 entries")
    return d


class Aligner:
    """Device-resident state of one alignment problem (pi_aligner)."""

    def __init__(self, geom1: Geometry, geom2: Geometry, kgrid: KGrid):
        self.geom1, self.geom2, self.kgrid = geom1, geom2, kgrid
        o1, o2 = _geom_obj(geom1), _geom_obj(geom2)
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().pi_aligner_create(ctypes.byref(o1), ctypes.byref(o2), kgrid.dirs.ctypes.data,
                                                kgrid.kmag.ctypes.data, kgrid.w.ctypes.data, kgrid.num_nodes,
                                                ctypes.byref(h)))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            _lib.lib().pi_aligner_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def fixed_volume(self) -> float:
        """Fourier self-volume of geometry 1 (the app's V1)."""
        v = ctypes.c_double(0.0)
        _lib.check(_lib.lib().pi_aligner_fixed_volume(self._h, ctypes.byref(v)))
        return float(v.value)

    def similarity(self, dofs2, measure=SIM_DICE, V1: float | None = None,
                   flags: int = SIM_FUNC_GRAD) -> SimilarityResult:
        d = _dofs12(dofs2)
        V1 = self.fixed_volume() if V1 is None else float(V1)
        val, sim = ctypes.c_double(0.0), ctypes.c_double(0.0)
        g = np.zeros(12) if flags & SIM_GRADIENT else None
        H = np.zeros((12, 12)) if flags & SIM_HESSIAN else None
        _lib.check(_lib.lib().pi_similarity(self._h, d.ctypes.data, _measure(measure), V1, int(flags),
                                            ctypes.byref(val), ctypes.byref(sim),
                                            g.ctypes.data if g is not None else None,
                                            H.ctypes.data if H is not None else None))
        return SimilarityResult(float(val.value), g, H, float(sim.value))

    def optimize(self, initial_dofs, measure=SIM_DICE, V1: float | None = None, tolerance: float = 1e-6,
                 max_iterations: int = 50, damping: float = 0.1) -> OptimizationState:
        d = _dofs12(initial_dofs)
        V1 = self.fixed_volume() if V1 is None else float(V1)
        st = _lib.OptimizationState()
        _lib.check(_lib.lib().pi_optimize_alignment(self._h, d.ctypes.data, _measure(measure), V1, float(tolerance),
                                                    int(max_iterations), float(damping), ctypes.byref(st)))
        return OptimizationState(np.array(st.dofs[:]), st.similarity, st.similarity_loss, st.iteration,
                                 bool(st.converged), st.status.decode(), st.steps, st.evaluations)


def compute_similarity(ref_geom1: Geometry, ref_geom2: Geometry, dofs2, kgrid: KGrid, measure, V1: float,
                       flags: int = SIM_FUNC_GRAD) -> SimilarityResult:
    """similarity_measure.hpp:37-48 (the AffineDoF argument is implied)."""
    with Aligner(ref_geom1, ref_geom2, kgrid) as a:
        return a.similarity(dofs2, measure, V1, flags)


def optimize_alignment(ref_geom1: Geometry, ref_geom2: Geometry, initial_dofs, kgrid: KGrid, measure, V1: float,
                       tolerance: float = 1e-6, max_iterations: int = 50, damping: float = 0.1) -> OptimizationState:
    """optimizer.hpp:22-33."""
    with Aligner(ref_geom1, ref_geom2, kgrid) as a:
        return a.optimize(initial_dofs, measure, V1, tolerance, max_iterations, damping)


def compute_moments(geom: Geometry, dofs=IDENTITY):
    """warm_start.hpp:17-24: (volume, centroid (3,), covariance (3, 3)).  Host only."""
    d = _dofs12(dofs)
    o = _geom_obj(geom)
    v = ctypes.c_double(0.0)
    c, C = np.zeros(3), np.zeros((3, 3))
    _lib.check(_lib.lib().pi_compute_moments(ctypes.byref(o), d.ctypes.data, ctypes.byref(v), c.ctypes.data,
                                             C.ctypes.data))
    return float(v.value), c, C


def compute_warm_start(geom1: Geometry, geom2: Geometry) -> np.ndarray:
    """warm_start.hpp:26-34: AffineDoF parameters aligning geometry 2's moments
    to geometry 1's (principal-axis signs canonicalised).  Host only."""
    o1, o2 = _geom_obj(geom1), _geom_obj(geom2)
    out = np.zeros(12)
    _lib.check(_lib.lib().pi_compute_warm_start(ctypes.byref(o1), ctypes.byref(o2), out.ctypes.data))
    return out


def moved(obj_geom: Geometry, dofs) -> SceneObject:
    """Geometry under an AffineDoF vector, as a SceneObject."""
    return SceneObject(obj_geom, _lib.DOF_AFFINE, _dofs12(dofs).copy())
