"""ctypes access to the test oracle.

TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg may use this module; the product library never does.

Two oracles:
  * ``Oracle``     -- oracle/sep_oracle.c, the C restatement of the reference
                      separation likelihood (builds everywhere with gcc);
  * ``Reference``  -- oracle/_ref/libmwref.so, the reference's own CPU sources
                      compiled by ``make -C oracle ref`` (only where the
                      reference sources are present).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libsep_oracle.so")
ORACLE_BIN = os.path.join(HERE, "_build", "sep_oracle")
REF_SO = os.path.join(HERE, "_ref", "libmwref.so")
REF_BIN = os.path.join(HERE, "_ref", "mw_ref")
REF_SRC = os.environ.get("MW_REFERENCE_DIR", "/root/reference")

_D = C.POINTER(C.c_double)


def build(reference: bool = True) -> None:
    """Compile the restatement, and the reference when its sources exist."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    if reference and os.path.isdir(os.path.join(REF_SRC, "milkyway_separation", "cpu")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_SRC}"], check=True)


def _arr(x):
    return np.ascontiguousarray(x, dtype=np.float64)


class Oracle:
    """One problem (parameter file + optional star file) in the restatement."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            if not os.path.exists(ORACLE_SO):
                build(reference=False)
            L = C.CDLL(ORACLE_SO)
            L.so_open.restype = C.c_void_p
            L.so_open.argtypes = [C.c_char_p, C.c_char_p]
            L.so_close.argtypes = [C.c_void_p]
            for f in ("so_n_theta", "so_n_streams", "so_n_areas", "so_n_stars", "so_convolve"):
                getattr(L, f).argtypes = [C.c_void_p]
                getattr(L, f).restype = C.c_int
            L.so_area_dims.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int)]
            L.so_evaluate.argtypes = [C.c_void_p, _D, C.c_int, C.c_int, _D, _D, _D, C.POINTER(C.c_int), _D,
                                      _D, _D]
            L.so_integrals.argtypes = [C.c_void_p, _D, C.c_int, C.c_int, _D, _D]
            L.so_likelihood.argtypes = [C.c_void_p, _D, _D, _D, C.POINTER(C.c_int), _D, _D, _D]
            L.so_cell_values.argtypes = [C.c_void_p, _D, C.c_int, _D]
            L.so_cell_lb.argtypes = [C.c_void_p, C.c_int, _D]
            L.so_r_tables.argtypes = [C.c_void_p, C.c_int, _D, _D, _D, _D, _D, _D]
            L.so_r_mag_tables.argtypes = [C.c_void_p, C.c_int, _D, _D]
            L.so_star_densities.argtypes = [C.c_void_p, _D, _D, _D]
            L.so_gauss_legendre.argtypes = [C.c_int, _D, _D]
            L.so_gc_to_lb.argtypes = [C.c_int, C.c_double, C.c_double, _D, _D]
            L.so_separation.argtypes = [C.c_void_p, _D, _D, _D, _D, _D]
            L.so_stripe_transform.argtypes = [C.c_int, C.c_int, _D]
            L.so_transform_point.argtypes = [_D, _D, _D]
            L.so_lbr_to_xyz.argtypes = [C.c_double, C.c_double, C.c_double, _D]
            cls._lib = L
        return cls._lib

    def __init__(self, param_path: str, star_path: str | None = None):
        L = self.lib()
        self._h = L.so_open(param_path.encode(), star_path.encode() if star_path else None)
        if not self._h:
            raise ValueError(f"oracle could not load {param_path} / {star_path}")

    def close(self):
        if self._h:
            self.lib().so_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n_theta(self):
        return self.lib().so_n_theta(self._h)

    @property
    def n_streams(self):
        return self.lib().so_n_streams(self._h)

    @property
    def n_areas(self):
        return self.lib().so_n_areas(self._h)

    @property
    def n_stars(self):
        return self.lib().so_n_stars(self._h)

    def area_dims(self, a):
        out = (C.c_int * 3)()
        self.lib().so_area_dims(self._h, a, out)
        return tuple(out)

    def evaluate(self, theta, rank: int = 0, nranks: int = 1) -> dict:
        S, A = self.n_streams, self.n_areas
        t = _arr(theta)
        areas = np.zeros(A * (1 + S))
        ints = np.zeros(1 + S)
        ps = C.c_double()
        nz = C.c_int()
        ll = C.c_double()
        bo = C.c_double()
        so = np.zeros(max(S, 1))
        rc = self.lib().so_evaluate(self._h, t.ctypes.data_as(_D), rank, nranks, areas.ctypes.data_as(_D),
                                    ints.ctypes.data_as(_D), C.byref(ps), C.byref(nz), C.byref(ll),
                                    C.byref(bo), so.ctypes.data_as(_D))
        if rc:
            raise RuntimeError("oracle evaluation failed")
        return {"background_integral": ints[0], "stream_integrals": list(ints[1:]),
                "area_integrals": areas.reshape(A, 1 + S).tolist(), "prob_sum": ps.value,
                "num_zero": nz.value, "likelihood": ll.value, "background_only_likelihood": bo.value,
                "stream_only_likelihood": list(so[:S])}

    def integrals(self, theta, rank: int = 0, nranks: int = 1):
        S, A = self.n_streams, self.n_areas
        t = _arr(theta)
        areas = np.zeros(A * (1 + S))
        ints = np.zeros(1 + S)
        self.lib().so_integrals(self._h, t.ctypes.data_as(_D), rank, nranks, areas.ctypes.data_as(_D),
                                ints.ctypes.data_as(_D))
        return ints, areas.reshape(A, 1 + S)

    def cell_values(self, theta, area: int = 0) -> np.ndarray:
        m, n, r = self.area_dims(area)
        out = np.zeros(m * n * r * (1 + self.n_streams))
        self.lib().so_cell_values(self._h, _arr(theta).ctypes.data_as(_D), area, out.ctypes.data_as(_D))
        return out.reshape(m, n, r, 1 + self.n_streams)

    def cell_lb(self, area: int = 0) -> np.ndarray:
        m, n, _ = self.area_dims(area)
        out = np.zeros(m * n * 2)
        self.lib().so_cell_lb(self._h, area, out.ctypes.data_as(_D))
        return out.reshape(m, n, 2)

    def star_densities(self, theta):
        N, S = self.n_stars, self.n_streams
        bg = np.zeros(N)
        st = np.zeros(max(N * S, 1))
        self.lib().so_star_densities(self._h, _arr(theta).ctypes.data_as(_D), bg.ctypes.data_as(_D),
                                     st.ctypes.data_as(_D))
        return bg, st[: N * S].reshape(N, S)

    def separation(self, theta, integrals):
        """(sprob [N][S], xyz [N][3], expected [S]) of separation.c."""
        N, S = self.n_stars, self.n_streams
        sp = np.zeros(max(N * S, 1))
        xyz = np.zeros(N * 3)
        ex = np.zeros(max(S, 1))
        self.lib().so_separation(self._h, _arr(theta).ctypes.data_as(_D), _arr(integrals).ctypes.data_as(_D),
                                 sp.ctypes.data_as(_D), xyz.ctypes.data_as(_D), ex.ctypes.data_as(_D))
        return sp[: N * S].reshape(N, S), xyz.reshape(N, 3), ex[:S]

    @classmethod
    def stripe_transform(cls, sgr, wedge):
        m = np.zeros(9)
        cls.lib().so_stripe_transform(sgr, wedge, m.ctypes.data_as(_D))
        return m.reshape(3, 3)

    @classmethod
    def transform_point(cls, xyz, mat):
        out = np.zeros(3)
        cls.lib().so_transform_point(_arr(xyz).ctypes.data_as(_D), _arr(mat).ravel().ctypes.data_as(_D),
                                     out.ctypes.data_as(_D))
        return out

    @classmethod
    def gauss_legendre(cls, n: int):
        x = np.zeros(n)
        w = np.zeros(n)
        cls.lib().so_gauss_legendre(n, x.ctypes.data_as(_D), w.ctypes.data_as(_D))
        return x, w

    @classmethod
    def gc_to_lb(cls, wedge, mu, nu):
        l = C.c_double()
        b = C.c_double()
        cls.lib().so_gc_to_lb(wedge, mu, nu, C.byref(l), C.byref(b))
        return l.value, b.value

    @classmethod
    def lbr_to_xyz(cls, l, b, r):
        out = np.zeros(3)
        cls.lib().so_lbr_to_xyz(l, b, r, out.ctypes.data_as(_D))
        return out


def reference_available() -> bool:
    return os.path.exists(REF_SO)


class Reference:
    """The reference's own CPU evaluator (oracle/_ref/libmwref.so)."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            L = C.CDLL(REF_SO)
            L.mwref_evaluate_files.argtypes = [C.c_char_p, C.c_char_p, _D, C.c_int, C.c_int, C.c_int, C.c_int,
                                               _D, _D, _D, _D, C.POINTER(C.c_int), _D, _D]
            L.mwref_evaluate_files.restype = C.c_int
            cls._lib = L
        return cls._lib

    @classmethod
    def stripe_transform(cls, sgr, wedge):
        """stripe_normal / sgr_stripe_normal + get_transform, from the
        reference's own compiled sources."""
        L = cls.lib()
        n = np.zeros(3)
        (L.sgr_stripe_normal if sgr else L.stripe_normal)(C.c_int(wedge), n.ctypes.data_as(_D))
        rows = [np.zeros(3) for _ in range(3)]
        mat = (_D * 3)(*[r.ctypes.data_as(_D) for r in rows])
        t = np.array([0.0, 0.0, 1.0])
        L.get_transform(n.ctypes.data_as(_D), t.ctypes.data_as(_D), mat)
        return np.array(rows)

    @classmethod
    def transform_point(cls, xyz, mat):
        """The reference's transform_point (stVector.c:155-169)."""
        L = cls.lib()
        rows = [np.ascontiguousarray(mat[i], dtype=np.float64) for i in range(3)]
        cm = (_D * 3)(*[r.ctypes.data_as(_D) for r in rows])
        p = _arr(xyz).copy()
        sun = np.array([-8.5, 0.0, 0.0])
        out = np.zeros(3)
        L.transform_point(p.ctypes.data_as(_D), cm, sun.ctypes.data_as(_D), out.ctypes.data_as(_D))
        return out

    @classmethod
    def invert_matrix(cls, a):
        """The reference's matrix_invert (util/matrix.c:298-319)."""
        L = cls.lib()
        a = np.ascontiguousarray(a, dtype=np.float64)
        n = a.shape[0]
        rows_in = [np.ascontiguousarray(a[i]) for i in range(n)]
        rows_out = [np.zeros(n) for _ in range(n)]
        pin = (_D * n)(*[r.ctypes.data_as(_D) for r in rows_in])
        pout = (_D * n)(*[r.ctypes.data_as(_D) for r in rows_out])
        L.matrix_invert.argtypes = [C.POINTER(_D), C.c_int, C.c_int, C.POINTER(_D)]
        L.matrix_invert.restype = C.c_int
        if L.matrix_invert(pin, n, n, pout) != 0:
            raise ValueError("singular matrix")
        return np.array(rows_out)

    @classmethod
    def evaluate(cls, param_path, star_path, theta, n_streams, n_areas, rank=0, nranks=1, repeats=1):
        t = _arr(theta)
        bg = C.c_double()
        st = np.zeros(max(n_streams, 1))
        areas = np.zeros(n_areas * (1 + n_streams))
        ps = C.c_double()
        nz = C.c_int()
        ll = C.c_double()
        secs = C.c_double()
        rc = cls.lib().mwref_evaluate_files(param_path.encode(), star_path.encode(), t.ctypes.data_as(_D),
                                            t.size, rank, nranks, repeats, C.byref(bg),
                                            st.ctypes.data_as(_D), areas.ctypes.data_as(_D), C.byref(ps),
                                            C.byref(nz), C.byref(ll), C.byref(secs))
        if rc:
            raise RuntimeError(f"reference evaluation failed ({rc})")
        return {"background_integral": bg.value, "stream_integrals": list(st[:n_streams]),
                "area_integrals": areas.reshape(n_areas, 1 + n_streams).tolist(), "prob_sum": ps.value,
                "num_zero": nz.value, "likelihood": ll.value, "seconds": secs.value}
