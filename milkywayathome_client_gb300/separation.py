"""Python mirror of the reference separation client's evaluation interface.

The call sequence reads like worker() in the reference
(src/milkyway_client_app.c:197-288)::

    ap = AstronomyParameters.read("astronomy_parameters.txt")   # read_astronomy_parameters
    sp = StarPoints.read("stars.txt")                          # read_star_points
    es = EvaluationState(ap, sp)                               # initialize_state
    assert len(theta) == ap.optimized_parameter_count          # :244-259
    likelihood = evaluate(theta, ap, es, sp) - 3.0             # :278

``evaluate`` is the plain FP64 GPU evaluator (``mwsep_evaluate``, an
EvalFunc); ``evaluate_mixed`` is the compensated-FP32 one.  ``Context``
exposes the resident-data API for many evaluations of one wedge.

Every compute call goes through libmwsep_gb300.so; there is no Python or CPU
implementation of the likelihood here.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from . import native as N


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class AstronomyParameters:
    """An ASTRONOMY_PARAMETERS owned by the library (cpu/parameters.h:37-71)."""

    def __init__(self):
        self._s = N.ASTRONOMY_PARAMETERS()
        self._owned = False

    @classmethod
    def read(cls, path: str) -> "AstronomyParameters":
        ap = cls()
        N.check(N.lib().mwsep_read_astronomy_parameters(str(path).encode(), C.byref(ap._s)),
                f"reading {path}")
        ap._owned = True
        return ap

    def write(self, path: str) -> None:
        N.check(N.lib().mwsep_write_astronomy_parameters(str(path).encode(), C.byref(self._s)),
                f"writing {path}")

    @classmethod
    def read_binary(cls, path: str) -> "AstronomyParameters":
        ap = cls()
        N.check(N.lib().mwsep_read_astronomy_parameters_binary(str(path).encode(), C.byref(ap._s)),
                f"reading {path}")
        ap._owned = True
        return ap

    def write_binary(self, path: str) -> None:
        N.check(N.lib().mwsep_write_astronomy_parameters_binary(str(path).encode(), C.byref(self._s)),
                f"writing {path}")

    def close(self) -> None:
        if self._owned:
            N.lib().mwsep_free_parameters(C.byref(self._s))
            self._owned = False

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def struct(self):
        return self._s

    @property
    def optimized_parameter_count(self) -> int:
        return N.lib().mwsep_get_optimized_parameter_count(C.byref(self._s))

    @property
    def number_streams(self) -> int:
        return self._s.number_streams

    @property
    def number_integrals(self) -> int:
        return self._s.number_integrals

    @property
    def convolve(self) -> int:
        return self._s.convolve

    def set_parameters(self, theta: Sequence[float]) -> None:
        t = np.ascontiguousarray(theta, dtype=np.float64)
        if t.size != self.optimized_parameter_count:
            raise ValueError(f"theta has {t.size} values, {self.optimized_parameter_count} expected")
        N.check(N.lib().mwsep_set_astronomy_parameters(C.byref(self._s), _dptr(t)))

    def search_parameters(self) -> np.ndarray:
        out = np.zeros(self.optimized_parameter_count)
        N.check(N.lib().mwsep_get_search_parameters(C.byref(self._s), _dptr(out)))
        return out

    def step(self) -> np.ndarray:
        """get_step: the step of each optimised parameter."""
        out = np.zeros(self.optimized_parameter_count)
        N.check(N.lib().mwsep_get_step(C.byref(self._s), _dptr(out)))
        return out

    def bounds(self):
        """(get_min_parameters, get_max_parameters)."""
        lo = np.zeros(self.optimized_parameter_count)
        hi = np.zeros(self.optimized_parameter_count)
        N.check(N.lib().mwsep_get_min_parameters(C.byref(self._s), _dptr(lo)))
        N.check(N.lib().mwsep_get_max_parameters(C.byref(self._s), _dptr(hi)))
        return lo, hi

    def split(self, rank: int, max_rank: int) -> None:
        N.check(N.lib().mwsep_split_astronomy_parameters(C.byref(self._s), rank, max_rank))

    def area(self, i: int) -> dict:
        a = self._s.integral[i].contents
        return {k: getattr(a, k) for k, _ in N.INTEGRAL._fields_}


class StarPoints:
    """A STAR_POINTS catalogue (cpu/star_points.h:27-31), rows (l, b, r_kpc)."""

    def __init__(self):
        self._s = N.STAR_POINTS()
        self._owned = False
        self._keep = None

    @classmethod
    def read(cls, path: str) -> "StarPoints":
        sp = cls()
        N.check(N.lib().mwsep_read_star_points(str(path).encode(), C.byref(sp._s)), f"reading {path}")
        sp._owned = True
        return sp

    @classmethod
    def from_array(cls, lbr: np.ndarray) -> "StarPoints":
        """Wrap an (N, 3) array without copying rows into C allocations."""
        a = np.ascontiguousarray(lbr, dtype=np.float64)
        if a.ndim != 2 or a.shape[1] != 3:
            raise ValueError("expected an (N, 3) array of l, b, r")
        n = a.shape[0]
        rows = (C.POINTER(C.c_double) * max(n, 1))()
        base = a.ctypes.data
        for i in range(n):
            rows[i] = C.cast(base + 24 * i, C.POINTER(C.c_double))
        sp = cls()
        sp._s.number_stars = n
        sp._s.stars = C.cast(rows, C.POINTER(C.POINTER(C.c_double)))
        sp._keep = (a, rows)
        return sp

    def write(self, path: str) -> None:
        N.check(N.lib().mwsep_write_star_points(str(path).encode(), C.byref(self._s)), f"writing {path}")

    @classmethod
    def read_binary(cls, path: str) -> "StarPoints":
        sp = cls()
        N.check(N.lib().mwsep_read_star_points_binary(str(path).encode(), C.byref(sp._s)), f"reading {path}")
        sp._owned = True
        return sp

    def write_binary(self, path: str) -> None:
        N.check(N.lib().mwsep_write_star_points_binary(str(path).encode(), C.byref(self._s)), f"writing {path}")

    def to_array(self) -> np.ndarray:
        n = self._s.number_stars
        out = np.empty((n, 3))
        for i in range(n):
            row = self._s.stars[i]
            out[i] = (row[0], row[1], row[2])
        return out

    def split(self, rank: int, max_rank: int) -> None:
        """Keep this rank's slice (split_star_points, cpu/star_points.c:105-131)."""
        if self._owned:
            N.check(N.lib().mwsep_split_star_points(C.byref(self._s), rank, max_rank))
            return
        if rank == 0 and max_rank == 0:
            return
        n = self.number_stars
        first = int(float(n) * (float(rank) / float(max_rank)))
        last = int(float(n) * ((float(rank) + 1.0) / float(max_rank)))
        other = StarPoints.from_array(self.to_array()[first:last])
        self._s, self._keep = other._s, other._keep
        other._keep = None

    def close(self) -> None:
        if self._owned:
            N.lib().mwsep_free_star_points(C.byref(self._s))
            self._owned = False

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def struct(self):
        return self._s

    @property
    def number_stars(self) -> int:
        return self._s.number_stars


class EvaluationState:
    """An EVALUATION_STATE (cpu/evaluation_state.h:43-58)."""

    def __init__(self, ap: AstronomyParameters, sp: StarPoints):
        self._s = N.EVALUATION_STATE()
        N.check(N.lib().mwsep_initialize_state(C.byref(ap.struct), C.byref(sp.struct), C.byref(self._s)))
        self._owned = True

    def close(self):
        if self._owned:
            N.lib().mwsep_free_state(C.byref(self._s))
            self._owned = False

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def struct(self):
        return self._s

    @property
    def background_integral(self) -> float:
        return self._s.background_integral

    @property
    def stream_integrals(self) -> List[float]:
        return [self._s.stream_integrals[i] for i in range(self._s.number_streams)]

    @property
    def area_integrals(self) -> List[List[float]]:
        out = []
        for a in range(self._s.number_integrals):
            ia = self._s.integral[a].contents
            out.append([ia.background_integral] + [ia.stream_integrals[i] for i in range(ia.number_streams)])
        return out

    @property
    def prob_sum(self) -> float:
        return self._s.prob_sum

    @property
    def num_zero(self) -> int:
        return self._s.num_zero


def _evalfunc(fn, theta, ap, es, sp) -> float:
    t = np.ascontiguousarray(theta, dtype=np.float64)
    if t.size != ap.optimized_parameter_count:
        raise N.MwsepError(N.MWSEP_ERR_PARAM_COUNT, "evaluate")
    v = fn(_dptr(t), C.byref(ap.struct), C.byref(es.struct), C.byref(sp.struct))
    if v != v:  # NaN: the library recorded why
        raise N.MwsepError(N.lib().mwsep_last_error(), "evaluate")
    return v


def evaluate(theta, ap: AstronomyParameters, es: EvaluationState, sp: StarPoints) -> float:
    """Plain FP64 GPU evaluation; returns prob_sum/N like cpu_evaluate
    (cpu/evaluation_optimized.c:756-784).  Subtract 3.0 for the likelihood."""
    return _evalfunc(N.lib().mwsep_evaluate, theta, ap, es, sp)


def integral_f(theta, ap: AstronomyParameters, es: EvaluationState, sp: StarPoints) -> List[float]:
    """integral_f (cpu/astronomy_worker.c:33-64) on the GPU: this rank's
    cut-subtracted background and stream integrals."""
    t = np.ascontiguousarray(theta, dtype=np.float64)
    out = np.zeros(1 + ap.number_streams)
    N.lib().mwsep_integral_f(_dptr(t), _dptr(out), C.byref(ap.struct), C.byref(es.struct), C.byref(sp.struct))
    if np.isnan(out).any():
        raise N.MwsepError(N.lib().mwsep_last_error(), "integral_f")
    return out.tolist()


def likelihood_f(integrals, ap: AstronomyParameters, es: EvaluationState, sp: StarPoints) -> List[float]:
    """likelihood_f (cpu/astronomy_worker.c:94-121) on the GPU: [prob_sum,
    bad_jacobians] of this rank's stars against the given integrals."""
    i = np.ascontiguousarray(integrals, dtype=np.float64)
    out = np.zeros(2)
    N.lib().mwsep_likelihood_f(_dptr(i), _dptr(out), C.byref(ap.struct), C.byref(es.struct), C.byref(sp.struct))
    if np.isnan(out).any():
        raise N.MwsepError(N.lib().mwsep_last_error(), "likelihood_f")
    return out.tolist()


def evaluate_mixed(theta, ap: AstronomyParameters, es: EvaluationState, sp: StarPoints) -> float:
    """Compensated-FP32 GPU evaluation with the same contract as evaluate."""
    return _evalfunc(N.lib().mwsep_evaluate_mixed, theta, ap, es, sp)


def evaluate_df(theta, ap: AstronomyParameters, es: EvaluationState, sp: StarPoints) -> float:
    """Double-float GPU evaluation (the plain form's bounds) with the same
    contract as evaluate."""
    return _evalfunc(N.lib().mwsep_evaluate_df, theta, ap, es, sp)


@dataclass
class Result:
    likelihood: float
    prob_sum: float
    num_zero: int
    background_integral: float
    stream_integrals: List[float]
    area_integrals: List[List[float]]
    background_only_likelihood: float
    stream_only_likelihood: List[float]

    @classmethod
    def from_c(cls, r: N.mwsep_result) -> "Result":
        S, A = r.number_streams, r.number_integrals
        return cls(
            likelihood=r.likelihood, prob_sum=r.prob_sum, num_zero=r.num_zero,
            background_integral=r.background_integral,
            stream_integrals=[r.stream_integrals[i] for i in range(S)],
            area_integrals=[[r.area_integrals[a][k] for k in range(1 + S)] for a in range(A)],
            background_only_likelihood=r.background_only_likelihood,
            stream_only_likelihood=[r.stream_only_likelihood[i] for i in range(S)],
        )

    @property
    def integrals(self) -> List[float]:
        return [self.background_integral] + list(self.stream_integrals)


class Context:
    """A device context with a resident wedge and catalogue (mwsep_ctx_*)."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        self._n_streams = 0
        self._n_stars = 0
        N.check(N.lib().mwsep_ctx_create(device, C.byref(self._h)), "mwsep_ctx_create")

    def close(self):
        if self._h:
            N.lib().mwsep_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_problem(self, ap: AstronomyParameters) -> None:
        N.check(N.lib().mwsep_ctx_set_problem(self._h, C.byref(ap.struct)), "set_problem")
        self._n_streams = ap.number_streams

    def set_stars(self, sp) -> None:
        if isinstance(sp, StarPoints):
            N.check(N.lib().mwsep_ctx_set_stars(self._h, C.byref(sp.struct)), "set_stars")
            self._n_stars = sp.number_stars
        else:
            a = np.asarray(sp, dtype=np.float64)
            l = np.ascontiguousarray(a[:, 0])
            b = np.ascontiguousarray(a[:, 1])
            r = np.ascontiguousarray(a[:, 2])
            N.check(N.lib().mwsep_ctx_set_stars_soa(self._h, a.shape[0], _dptr(l), _dptr(b), _dptr(r)),
                    "set_stars")
            self._n_stars = a.shape[0]

    def set_stars_file(self, path: str) -> None:
        """A binary catalogue (mapped) or the reference's text star file."""
        N.check(N.lib().mwsep_ctx_set_stars_file(self._h, str(path).encode()), "set_stars_file")
        self._n_stars = self._probe_stars(path)

    @staticmethod
    def _probe_stars(path: str) -> int:
        with open(path, "rb") as f:
            head = f.read(24)
        if head[:8] == b"MWSEPCAT":
            return int.from_bytes(head[16:24], "little")
        with open(path) as f:
            return int(f.readline().split()[0])

    @property
    def theta_count(self) -> int:
        return N.lib().mwsep_ctx_theta_count(self._h)

    def evaluate(self, theta, precision: int = N.MWSEP_PLAIN_F64) -> Result:
        t = np.ascontiguousarray(theta, dtype=np.float64)
        if t.size != self.theta_count:
            raise N.MwsepError(N.MWSEP_ERR_PARAM_COUNT, "evaluate")
        r = N.mwsep_result()
        N.check(N.lib().mwsep_ctx_evaluate(self._h, _dptr(t), precision, C.byref(r)), "evaluate")
        return Result.from_c(r)

    def integrals(self, theta, precision: int = N.MWSEP_PLAIN_F64) -> Result:
        """The integrals alone of the resident problem's cells
        (mwsep_ctx_integrals): a rank's integral_f."""
        t = np.ascontiguousarray(theta, dtype=np.float64)
        r = N.mwsep_result()
        N.check(N.lib().mwsep_ctx_integrals(self._h, _dptr(t), precision, C.byref(r)), "integrals")
        return Result.from_c(r)

    def likelihood(self, theta, integrals, precision: int = N.MWSEP_PLAIN_F64) -> Result:
        """The resident catalogue's likelihood against given cut-subtracted
        integrals (mwsep_ctx_likelihood): a rank's likelihood_f."""
        t = np.ascontiguousarray(theta, dtype=np.float64)
        i = np.ascontiguousarray(integrals, dtype=np.float64)
        r = N.mwsep_result()
        N.check(N.lib().mwsep_ctx_likelihood(self._h, _dptr(t), _dptr(i), precision, C.byref(r)), "likelihood")
        return Result.from_c(r)

    def evaluate_batch(self, thetas, precision: int = N.MWSEP_PLAIN_F64) -> List[Result]:
        t = np.ascontiguousarray(thetas, dtype=np.float64)
        if t.ndim != 2 or t.shape[1] != self.theta_count:
            raise N.MwsepError(N.MWSEP_ERR_PARAM_COUNT, "evaluate_batch")
        out = (N.mwsep_result * t.shape[0])()
        N.check(N.lib().mwsep_ctx_evaluate_batch(self._h, t.shape[0], _dptr(t), precision, out),
                "evaluate_batch")
        return [Result.from_c(out[i]) for i in range(t.shape[0])]

    @property
    def device_bytes(self) -> int:
        v = C.c_size_t()
        N.check(N.lib().mwsep_ctx_device_bytes(self._h, C.byref(v)))
        return v.value

    def last_timings(self) -> dict:
        a = (C.c_double * 5)()
        N.check(N.lib().mwsep_ctx_last_timings(self._h, a))
        return {"integral_ms": a[0], "integral_reduce_ms": a[1], "likelihood_ms": a[2],
                "likelihood_reduce_ms": a[3], "total_ms": a[4]}

    # ---- many resident wedges (the tiled engine) ----
    def add_wedge(self, ap: AstronomyParameters, sp: StarPoints) -> int:
        wid = C.c_int()
        N.check(N.lib().mwsep_ctx_add_wedge(self._h, C.byref(ap.struct), C.byref(sp.struct), C.byref(wid)),
                "add_wedge")
        return wid.value

    def wedge_theta_count(self, wedge: int) -> int:
        return N.lib().mwsep_ctx_wedge_theta_count(self._h, wedge)

    def wedge_points(self, wedge: int) -> float:
        """Density points one evaluation of the wedge computes."""
        v = C.c_double()
        N.check(N.lib().mwsep_ctx_wedge_points(self._h, wedge, C.byref(v)))
        return v.value

    def wedge_bytes(self, wedge: int) -> int:
        v = C.c_size_t()
        N.check(N.lib().mwsep_ctx_wedge_bytes(self._h, wedge, C.byref(v)))
        return v.value

    def set_hbm_budget(self, nbytes: int) -> None:
        N.check(N.lib().mwsep_ctx_set_hbm_budget(self._h, nbytes))

    def evaluate_requests(self, requests, precision: int = N.MWSEP_PLAIN_F64) -> List[Result]:
        """requests: sequence of (wedge_id, theta)."""
        keep = []
        arr = (N.mwsep_request * len(requests))()
        for i, (w, t) in enumerate(requests):
            a = np.ascontiguousarray(t, dtype=np.float64)
            if a.size != self.wedge_theta_count(w):
                raise N.MwsepError(N.MWSEP_ERR_PARAM_COUNT, "evaluate_requests")
            keep.append(a)
            arr[i].wedge = w
            arr[i].theta = _dptr(a)
        out = (N.mwsep_result * len(requests))()
        N.check(N.lib().mwsep_ctx_evaluate_requests(self._h, len(requests), arr, precision, out),
                "evaluate_requests")
        return [Result.from_c(out[i]) for i in range(len(requests))]

    def autotune(self, wedge: int, precision: int) -> float:
        ms = C.c_double()
        N.check(N.lib().mwsep_ctx_autotune(self._h, wedge, precision, C.byref(ms)), "autotune")
        return ms.value

    def tile_shape(self, wedge: int, precision: int):
        kc, ti = C.c_int(), C.c_int()
        N.check(N.lib().mwsep_ctx_wedge_tile_shape(self._h, wedge, precision, C.byref(kc), C.byref(ti)))
        return kc.value, ti.value

    def last_launches(self) -> int:
        v = C.c_int()
        N.check(N.lib().mwsep_ctx_last_launches(self._h, C.byref(v)))
        return v.value

    def gradient(self, wedge: int, theta, step, precision: int = N.MWSEP_PLAIN_F64):
        """(f0, gradient) by central differences, one engine batch."""
        t = np.ascontiguousarray(theta, dtype=np.float64)
        h = np.ascontiguousarray(step, dtype=np.float64)
        if t.size != h.size:
            raise ValueError("theta and step differ in length")
        f0 = C.c_double()
        g = np.zeros(t.size)
        N.check(N.lib().mwsep_ctx_gradient(self._h, wedge, _dptr(t), _dptr(h), precision, C.byref(f0), _dptr(g)),
                "gradient")
        return f0.value, g

    def hessian(self, wedge: int, theta, step, precision: int = N.MWSEP_PLAIN_F64):
        """(f0, gradient, hessian) by central differences (2P^2+1 evaluations)."""
        t = np.ascontiguousarray(theta, dtype=np.float64)
        h = np.ascontiguousarray(step, dtype=np.float64)
        if t.size != h.size:
            raise ValueError("theta and step differ in length")
        f0 = C.c_double()
        g = np.zeros(t.size)
        H = np.zeros((t.size, t.size))
        N.check(N.lib().mwsep_ctx_hessian(self._h, wedge, _dptr(t), _dptr(h), precision, C.byref(f0), _dptr(g),
                                          _dptr(H)), "hessian")
        return f0.value, g, H

    def separation(self, theta, seed: int = 0) -> dict:
        """Separate the catalogue at theta (cpu/separation.c:37-254).

        Returns sprob [N][S], assignment [N] (0 background, k stream k),
        xyz [N][3] in the stripe frame, expected [S], assigned [S],
        background_assigned, the integrals and the likelihood."""
        t = np.ascontiguousarray(theta, dtype=np.float64)
        if t.size != self.theta_count:
            raise ValueError(f"theta has {t.size} values, the problem takes {self.theta_count}")
        sm = N.mwsep_separation_summary()
        n = self._n_stars
        s_count = self._n_streams
        sprob = np.zeros((n, max(s_count, 1)))
        assign = np.zeros(n, dtype=np.int32)
        xyz = np.zeros((n, 3))
        N.check(N.lib().mwsep_ctx_separation(self._h, _dptr(t), C.c_ulonglong(seed), _dptr(sprob),
                                             assign.ctypes.data_as(C.POINTER(C.c_int)), _dptr(xyz),
                                             C.byref(sm)), "separation")
        S = sm.number_streams
        return {"sprob": sprob[:, :S], "assignment": assign, "xyz": xyz, "expected": list(sm.expected[:S]),
                "assigned": list(sm.assigned[:S]), "background_assigned": sm.background_assigned,
                "background_integral": sm.background_integral, "stream_integrals": list(sm.stream_integrals[:S]),
                "likelihood": sm.likelihood}


class StarCatalogue:
    """A binary star catalogue mapped read-only; l, b, r are views into the
    mapping (valid until close)."""

    def __init__(self, path: str):
        self._c = N.mwsep_star_catalogue()
        N.check(N.lib().mwsep_map_star_catalogue(str(path).encode(), C.byref(self._c)), f"mapping {path}")
        n = self._c.number_stars
        self.number_stars = n
        self.l = np.ctypeslib.as_array(self._c.l, shape=(n,)) if n else np.zeros(0)
        self.b = np.ctypeslib.as_array(self._c.b, shape=(n,)) if n else np.zeros(0)
        self.r = np.ctypeslib.as_array(self._c.r, shape=(n,)) if n else np.zeros(0)

    @staticmethod
    def write(path: str, lbr) -> None:
        a = np.asarray(lbr, dtype=np.float64)
        cols = [np.ascontiguousarray(a[:, k]) for k in range(3)]
        N.check(N.lib().mwsep_write_star_catalogue(str(path).encode(), a.shape[0], *[_dptr(c) for c in cols]),
                f"writing {path}")

    def close(self) -> None:
        if self._c.map:
            self.l = self.b = self.r = None
            N.lib().mwsep_unmap_star_catalogue(C.byref(self._c))

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def invert_matrix(a) -> np.ndarray:
    """matrix_invert of util/matrix.c (LU with partial pivoting)."""
    m = np.ascontiguousarray(a, dtype=np.float64)
    out = np.zeros_like(m)
    N.check(N.lib().mwsep_invert_matrix(m.shape[0], _dptr(m), _dptr(out)), "invert_matrix")
    return out


def errors_from_hessian(hessian, number_stars: int):
    """errors() of cpu/errors.c: (sigma = H^-1 / N, sqrt|sigma_ii|)."""
    H = np.ascontiguousarray(hessian, dtype=np.float64)
    n = H.shape[0]
    sigma = np.zeros((n, n))
    sd = np.zeros(n)
    N.check(N.lib().mwsep_errors_from_hessian(n, _dptr(H), int(number_stars), _dptr(sigma), _dptr(sd)),
            "errors_from_hessian")
    return sigma, sd


def write_errors(path: str, hessian, sigma, stddev) -> None:
    H = np.ascontiguousarray(hessian, dtype=np.float64)
    S = np.ascontiguousarray(sigma, dtype=np.float64)
    d = np.ascontiguousarray(stddev, dtype=np.float64)
    N.check(N.lib().mwsep_write_errors(path.encode(), H.shape[0], _dptr(H), _dptr(S), _dptr(d)), "write_errors")


def write_separation(path: str, assignment, xyz) -> None:
    """Write separation()'s output file: "<stream> <x> <y> <z>" per star."""
    a = np.ascontiguousarray(assignment, dtype=np.int32)
    x = np.ascontiguousarray(xyz, dtype=np.float64)
    if x.shape != (a.size, 3):
        raise ValueError("xyz must be [N][3] for N assignments")
    N.check(N.lib().mwsep_write_separation(path.encode(), a.size, a.ctypes.data_as(C.POINTER(C.c_int)),
                                           _dptr(x)), "write_separation")


def stripe_transform(sgr_coordinates: int, wedge: int) -> np.ndarray:
    """Row-major 3x3 rotation taking the stripe's normal onto the z axis."""
    m = np.zeros(9)
    N.check(N.lib().mwsep_stripe_transform(int(sgr_coordinates), int(wedge), _dptr(m)), "stripe_transform")
    return m.reshape(3, 3)


class Server:
    """Continuous-batching server over a context's resident wedges
    (mwsep_server_*).  Add the wedges to the context first."""

    def __init__(self, ctx: Context, lanes: int = 2, max_batch: int = 256, lane_hbm_bytes: int = 0,
                 target_batch_ms: float = 0.0, max_queued: int = 0):
        cfg = N.mwsep_server_config(lanes, max_batch, lane_hbm_bytes, target_batch_ms, max_queued)
        self._h = C.c_void_p()
        self._ctx = ctx
        N.check(N.lib().mwsep_server_create(ctx._h, C.byref(cfg), C.byref(self._h)), "server_create")

    def submit(self, wedge: int, theta, precision: int = N.MWSEP_MIXED_F32) -> int:
        t = np.ascontiguousarray(theta, dtype=np.float64)
        if t.size != self._ctx.wedge_theta_count(wedge):
            raise N.MwsepError(N.MWSEP_ERR_PARAM_COUNT, "submit")
        rid = C.c_ulonglong()
        N.check(N.lib().mwsep_server_submit(self._h, wedge, _dptr(t), precision, C.byref(rid)), "submit")
        return rid.value

    def wait(self, rid: int, timeout: float = 60.0) -> Result:
        r = N.mwsep_result()
        N.check(N.lib().mwsep_server_wait(self._h, rid, timeout, C.byref(r)), "wait")
        return Result.from_c(r)

    def try_wait(self, rid: int, timeout: float):
        """(status, Result or None) without raising."""
        r = N.mwsep_result()
        st = N.lib().mwsep_server_wait(self._h, rid, timeout, C.byref(r))
        return st, (Result.from_c(r) if st == N.MWSEP_OK else None)

    def cancel(self, rid: int) -> int:
        return N.lib().mwsep_server_cancel(self._h, rid)

    def stats(self) -> dict:
        st = N.mwsep_server_stats()
        N.check(N.lib().mwsep_server_get_stats(self._h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in N.mwsep_server_stats._fields_}

    def reset_stats(self) -> None:
        N.check(N.lib().mwsep_server_reset_stats(self._h))

    def close(self) -> None:
        if self._h:
            N.lib().mwsep_server_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
