"""Seeded synthetic separation workloads written in the reference's file formats.

The reference measures on real survey wedges (its tests/ fixtures); the
workloads here are synthetic stand-ins with the benchmark shapes:

  config 0  mu [310,340] x 80, nu [-1.25,1.25] x 40, g [16,22.5] x 70,
            convolve 30, 1 stream, 10k stars                (CPU-runnable)
  config 1  mu [310,420] x 1600, nu x 640, g x 140, convolve 120,
            3 streams, 100k stars                            (full size)
  config 2  400 x 160 x 140, convolve 60, 3 streams, 50k stars, and a
            population of 256 parameter vectors
  config 3  6 wedges with log-uniform sizes, 1-4 streams, 20k-200k stars

Density model (cpu/evaluation_optimized.c:190-299): Hernquist-like halo with
alpha = delta = 1, q = 0.7, r0 = 6 kpc, Sun at x = -8.5 kpc; Gaussian tubes
with axis angles theta ~ U[0, pi), phi ~ U[0, 2 pi), centre mu offset
U[-5, 5] deg about the wedge centre at nu = 0, centre distance U[5, 40] kpc,
sigma ~ U[1, 4] kpc, weight epsilon ~ U[-3, 1].  Stars are drawn from that
mixture inside the wedge by rejection sampling in (mu, nu, g) and mapped to
(l, b) with the survey transform; g -> r uses the reference's mag2r,
r = 10^((g - 4.2)/5 + 1)/1000 kpc.  Everything derives from one PCG64 seed.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

DEG = 180.0 / math.pi


# ----------------------------------------------------------------- geometry
def _bound(a, lo, hi):
    a = np.where(a < lo, a + 360.0, a)
    a = np.where(a >= hi, a - 360.0, a)
    return a


def _bound2(theta, phi):
    theta = _bound(theta, -180.0, 180.0)
    flip = np.abs(theta) > 90.0
    theta = np.where(flip, 180.0 - theta, theta)
    phi = np.where(flip, phi + 180.0, phi)
    theta = _bound(theta, -180.0, 180.0)
    phi = _bound(phi, 0.0, 360.0)
    phi = np.where(np.abs(theta) == 90.0, 0.0, phi)
    return theta, phi


def wedge_incl(wedge: int) -> float:
    return wedge * 2.5 - 57.5 - (180.0 if wedge > 46 else 0.0) + 32.5


def gc_to_lb(wedge: int, mu, nu):
    """Survey great-circle (mu, nu) -> Galactic (l, b), degrees (vectorised;
    the survey transform of atSurveyGeometry.c:26-83)."""
    mu = np.asarray(mu, dtype=np.float64) * math.pi / 180.0
    nu = np.asarray(nu, dtype=np.float64) * math.pi / 180.0
    node = 95.0 * math.pi / 180.0
    inc = wedge_incl(wedge) * math.pi / 180.0
    x2 = np.cos(mu - node) * np.cos(nu)
    y2 = np.sin(mu - node) * np.cos(nu)
    z2 = np.sin(nu)
    y1 = y2 * math.cos(inc) - z2 * math.sin(inc)
    z1 = y2 * math.sin(inc) + z2 * math.cos(inc)
    ra = (np.arctan2(y1, x2) + node) * 180.0 / math.pi
    dec = np.arcsin(np.clip(z1, -1, 1)) * 180.0 / math.pi
    dec, ra = _bound2(dec, ra)
    ra = ra * math.pi / 180.0
    dec = dec * math.pi / 180.0
    m = np.array([[-0.054875539726, -0.873437108010, -0.483834985808],
                  [0.494109453312, -0.444829589425, 0.746982251810],
                  [-0.867666135858, -0.198076386122, 0.455983795705]])
    v = np.stack([np.cos(ra) * np.cos(dec), np.sin(ra) * np.cos(dec), np.sin(dec)])
    w = np.tensordot(m, v, axes=1)
    l = np.mod(np.arctan2(w[1], w[0]), 2 * math.pi) * 180.0 / math.pi
    b = np.arctan2(w[2], np.hypot(w[0], w[1])) * 180.0 / math.pi
    b, l = _bound2(b, l)
    return l, b


def mag2r(g):
    return 10.0 ** ((np.asarray(g) - 4.2) / 5.0 + 1.0) / 1000.0


def lbr_to_xyz(l, b, r):
    l = np.asarray(l) / DEG
    b = np.asarray(b) / DEG
    zp = r * np.cos(b)
    return np.stack([zp * np.cos(l) - 8.5, zp * np.sin(l), r * np.sin(b)], axis=-1)


# ----------------------------------------------------------------- problems
@dataclass
class Stream:
    weight: float
    mu: float
    r: float
    theta: float
    phi: float
    sigma: float


@dataclass
class Area:
    mu: tuple  # (min, max, steps)
    nu: tuple
    r: tuple


@dataclass
class Problem:
    """One wedge: everything the reference's astronomy_parameters file holds."""
    wedge: int = 82
    convolve: int = 30
    q: float = 0.7
    r0: float = 6.0
    alpha: float = 1.0
    delta: float = 1.0
    aux: Optional[tuple] = None          # (a, b, c) when aux_bg_profile = 1
    sgr: int = 0
    background_weight: float = 0.0
    streams: List[Stream] = field(default_factory=list)
    areas: List[Area] = field(default_factory=list)
    optimize_alpha_delta: bool = False

    # ---- theta layout: q, r0 (+ alpha, delta) (+ aux a, b, c), then per stream
    #      weight, mu, r, theta, phi, sigma (cpu/parameters.c:332-363)
    def theta(self) -> np.ndarray:
        t = []
        if self.optimize_alpha_delta:
            t.append(self.alpha)
        t += [self.q, self.r0]
        if self.optimize_alpha_delta:
            t.append(self.delta)
        if self.aux is not None:
            t += list(self.aux)
        for s in self.streams:
            t += [s.weight, s.mu, s.r, s.theta, s.phi, s.sigma]
        return np.array(t, dtype=np.float64)

    def bounds(self):
        lo, hi = [], []
        if self.optimize_alpha_delta:
            lo.append(0.0); hi.append(3.0)
        lo += [0.3, 1.0]; hi += [1.0, 30.0]
        if self.optimize_alpha_delta:
            lo.append(0.1); hi.append(3.0)
        if self.aux is not None:
            lo += [-1000.0] * 3; hi += [1000.0] * 3
        mu0, mu1 = self.areas[0].mu[0], self.areas[0].mu[1]
        for _ in self.streams:
            lo += [-20.0, mu0, 2.3, 0.0, 0.0, 1.0]
            hi += [20.0, mu1, 45.7, 2 * math.pi, 2 * math.pi, 20.0]
        return np.array(lo), np.array(hi)

    def cells(self) -> int:
        return sum(a.mu[2] * a.nu[2] * a.r[2] for a in self.areas)

    def write(self, path: str) -> None:
        """astronomy_parameters text (cpu/parameters.c:230-305 layout)."""
        bg = [self.alpha, self.q, self.r0, self.delta]
        opt = [1 if self.optimize_alpha_delta else 0, 1, 1, 1 if self.optimize_alpha_delta else 0]
        step = [0.02, 0.1, 0.1, 0.02]
        bmin = [0.0, 0.3, 1.0, 0.1]
        bmax = [3.0, 1.0, 30.0, 3.0]
        if self.aux is not None:
            bg += list(self.aux)
            opt += [1, 1, 1]
            step += [1, 1, 1]
            bmin += [-1000, -1000, -1000]
            bmax += [1000, 1000, 1000]
        lo, hi = self.bounds()

        def arr(name, xs, fmt="%.20f"):
            return f"{name}[{len(xs)}]: " + ", ".join(fmt % x for x in xs) + "\n"

        mu0, mu1 = self.areas[0].mu[0], self.areas[0].mu[1]
        with open(path, "w") as f:
            f.write("parameters_version: 0.04\n")
            f.write(f"number_parameters: {len(bg)}\n")
            f.write("background_weight: %.6f\n" % self.background_weight)
            f.write(arr("background_parameters", bg))
            f.write(arr("background_step", step))
            f.write(arr("background_min", bmin))
            f.write(arr("background_max", bmax))
            f.write(f"optimize_parameter[{len(opt)}]: " + ", ".join(str(o) for o in opt) + "\n")
            f.write(f"number_streams: {len(self.streams)}, 5\n")
            for s in self.streams:
                f.write("stream_weight: %.20f\n" % s.weight)
                f.write("stream_weight_step: 0.1\n")
                f.write("stream_weight_min: -20.0\n")
                f.write("stream_weight_max: 20.0\n")
                f.write("optimize_weight: 1\n")
                f.write(arr("stream_parameters", [s.mu, s.r, s.theta, s.phi, s.sigma]))
                f.write(arr("stream_step", [0.3] * 5))
                f.write(arr("stream_min", [mu0, 2.3, 0.0, 0.0, 1.0]))
                f.write(arr("stream_max", [mu1, 45.7, 2 * math.pi, 2 * math.pi, 20.0]))
                f.write("optimize_parameter[5]: 1, 1, 1, 1, 1\n")
            f.write(f"convolve: {self.convolve}\n")
            f.write(f"sgr_coordinates: {self.sgr}\n")
            f.write(f"aux_bg_profile: {1 if self.aux is not None else 0}\n")
            f.write(f"wedge: {self.wedge}\n")
            a = self.areas[0]
            f.write("r[min,max,steps]: %.10f, %.10f, %d\n" % a.r)
            f.write("mu[min,max,steps]: %.10f, %.10f, %d\n" % a.mu)
            f.write("nu[min,max,steps]: %.10f, %.10f, %d\n" % a.nu)
            f.write(f"number_cuts: {len(self.areas) - 1}\n")
            for c in self.areas[1:]:
                f.write("r_cut[min,max,steps][3]: %.10f, %.10f, %d\n" % c.r)
                f.write("mu_cut[min,max,steps][3]: %.10f, %.10f, %d\n" % c.mu)
                f.write("nu_cut[min,max,steps][3]: %.10f, %.10f, %d\n" % c.nu)


def draw_streams(rng, n, mu_lo, mu_hi) -> List[Stream]:
    centre = 0.5 * (mu_lo + mu_hi)
    out = []
    for _ in range(n):
        out.append(Stream(weight=float(rng.uniform(-3.0, 1.0)),
                          mu=float(centre + rng.uniform(-5.0, 5.0)),
                          r=float(rng.uniform(5.0, 40.0)),
                          theta=float(rng.uniform(0.0, math.pi)),
                          phi=float(rng.uniform(0.0, 2 * math.pi)),
                          sigma=float(rng.uniform(1.0, 4.0))))
    return out


# ----------------------------------------------------------------- catalogue
def _component_density(p: Problem, comp: int, mu, nu, g):
    """Unconvolved density of one mixture component times the volume element
    r^3 cos(nu) (per unit mu, nu, g) and the detection efficiency."""
    l, b = gc_to_lb(p.wedge, mu, nu)
    r = mag2r(g)
    x = lbr_to_xyz(l, b, r)
    jac = r ** 3 * np.cos(np.asarray(nu) / DEG)
    eff = 0.9402 / (np.exp(1.6171 * (np.asarray(g) - 23.5877)) + 1.0)
    if comp == 0:
        rg = np.sqrt(x[..., 0] ** 2 + x[..., 1] ** 2 + (x[..., 2] / p.q) ** 2)
        rho = 1.0 / (rg * (rg + p.r0) ** 3)
    else:
        s = p.streams[comp - 1]
        cl, cb = gc_to_lb(p.wedge, s.mu, 0.0)
        c = lbr_to_xyz(cl, cb, s.r)
        a = np.array([math.sin(s.theta) * math.cos(s.phi), math.sin(s.theta) * math.sin(s.phi),
                      math.cos(s.theta)])
        d = x - c
        d = d - (d @ a)[..., None] * a
        rho = np.exp(-np.sum(d * d, axis=-1) / (2 * s.sigma ** 2))
    return rho * jac * eff


def sample_stars(p: Problem, n: int, rng) -> np.ndarray:
    """Rejection-sample n stars (l, b, r_kpc) from the mixture inside area 0."""
    a = p.areas[0]
    mu0, mu1 = a.mu[0], a.mu[1]
    nu0, nu1 = a.nu[0], a.nu[1]
    g0, g1 = a.r[0], a.r[1]
    # a stream the model switches off (|sigma| < 1e-4, cpu/evaluation_optimized.c:279-280)
    # contributes no stars
    w = np.array([math.exp(p.background_weight)] +
                 [0.0 if abs(s.sigma) < 1e-4 else math.exp(s.weight) for s in p.streams])
    counts = rng.multinomial(n, w / w.sum())
    # piecewise-constant envelope on a coarse grid
    G = (48, 12, 48)
    gm = np.linspace(mu0, mu1, G[0] + 1)
    gn = np.linspace(nu0, nu1, G[1] + 1)
    gg = np.linspace(g0, g1, G[2] + 1)
    M, Nn, Gg = np.meshgrid(gm, gn, gg, indexing="ij")
    out = []
    order = list(range(1, len(counts))) + [0]
    for comp in order:
        cnt = int(counts[comp])
        if cnt == 0:
            continue
        corner = _component_density(p, comp, M, Nn, Gg)
        # envelope per cell: 2x the max over its 8 corners (plus a floor)
        env = np.maximum.reduce([corner[i:i + G[0], j:j + G[1], k:k + G[2]]
                                 for i in (0, 1) for j in (0, 1) for k in (0, 1)]) * 2.0
        if not np.isfinite(env).all() or env.max() <= 0.0:
            counts[0] += cnt  # no support inside the wedge: give the stars to the halo
            continue
        env = np.maximum(env, env.max() * 1e-6)
        prob = env.ravel() / env.sum()
        got = []
        need = cnt
        guard = 0
        while need > 0 and guard < 200:
            guard += 1
            m = max(4 * need, 1024)
            cell = rng.choice(prob.size, size=m, p=prob)
            ci, cj, ck = np.unravel_index(cell, env.shape)
            mu = gm[ci] + rng.uniform(size=m) * (gm[1] - gm[0])
            nu = gn[cj] + rng.uniform(size=m) * (gn[1] - gn[0])
            g = gg[ck] + rng.uniform(size=m) * (gg[1] - gg[0])
            dens = _component_density(p, comp, mu, nu, g)
            acc = rng.uniform(size=m) * env[ci, cj, ck] < dens
            idx = np.nonzero(acc)[0][:need]
            if idx.size:
                got.append(np.stack([mu[idx], nu[idx], g[idx]], axis=1))
                need -= idx.size
        if need > 0:  # envelope far too loose: fill uniformly (never hit in practice)
            mu = rng.uniform(mu0, mu1, need)
            nu = rng.uniform(nu0, nu1, need)
            g = rng.uniform(g0, g1, need)
            got.append(np.stack([mu, nu, g], axis=1))
        out.append(np.concatenate(got))
    mng = np.concatenate(out)
    mng = mng[rng.permutation(mng.shape[0])]
    l, b = gc_to_lb(p.wedge, mng[:, 0], mng[:, 1])
    r = mag2r(mng[:, 2])
    return np.stack([l, b, r], axis=1)


def write_stars(path: str, lbr: np.ndarray) -> None:
    """Star file (cpu/star_points.c:83-93): count, then "%lf %lf %lf" rows."""
    with open(path, "w") as f:
        f.write(f"{lbr.shape[0]}\n")
        np.savetxt(f, lbr, fmt="%f %f %f")


def read_stars(path: str) -> np.ndarray:
    with open(path) as f:
        n = int(f.readline())
        if n == 0:
            return np.zeros((0, 3))
        a = np.loadtxt(f, dtype=np.float64, ndmin=2)
    return a[:n]


# ----------------------------------------------------------------- configs
CONFIG_SEED_BASE = 0


def config(idx: int) -> dict:
    """Problem(s), catalogue size(s) and theta vector(s) of a benchmark config."""
    rng = np.random.Generator(np.random.PCG64(CONFIG_SEED_BASE + idx))
    if idx == 0:
        p = Problem(convolve=30, areas=[Area((310.0, 340.0, 80), (-1.25, 1.25, 40), (16.0, 22.5, 70))])
        p.streams = draw_streams(rng, 1, 310.0, 340.0)
        return {"problems": [p], "stars": [10_000], "rng": rng}
    if idx == 1:
        p = Problem(convolve=120, areas=[Area((310.0, 420.0, 1600), (-1.25, 1.25, 640), (16.0, 22.5, 140))])
        p.streams = draw_streams(rng, 3, 310.0, 420.0)
        return {"problems": [p], "stars": [100_000], "rng": rng}
    if idx == 2:
        p = Problem(convolve=60, areas=[Area((310.0, 420.0, 400), (-1.25, 1.25, 160), (16.0, 22.5, 140))])
        p.streams = draw_streams(rng, 3, 310.0, 420.0)
        base = p.theta()
        lo, hi = p.bounds()
        pert = rng.normal(0.0, 0.05 * (hi - lo), size=(256, base.size))
        thetas = np.clip(base + pert, lo, hi)
        return {"problems": [p], "stars": [50_000], "thetas": thetas, "rng": rng}
    if idx == 3:
        probs, stars = [], []
        for _ in range(6):
            mu_steps = int(round(math.exp(rng.uniform(math.log(200), math.log(1600)))))
            nu_steps = int(round(math.exp(rng.uniform(math.log(80), math.log(640)))))
            r_steps = int(round(math.exp(rng.uniform(math.log(70), math.log(700)))))
            conv = int(round(math.exp(rng.uniform(math.log(30), math.log(120)))))
            S = int(rng.integers(1, 5))
            n = int(round(math.exp(rng.uniform(math.log(20_000), math.log(200_000)))))
            p = Problem(convolve=conv, areas=[Area((310.0, 420.0, mu_steps), (-1.25, 1.25, nu_steps),
                                                   (16.0, 22.5, r_steps))])
            p.streams = draw_streams(rng, S, 310.0, 420.0)
            probs.append(p)
            stars.append(n)
        return {"problems": probs, "stars": stars, "rng": rng}
    raise ValueError(f"no config {idx}")


def materialise(idx: int, out_dir: str, star_scale: float = 1.0) -> dict:
    """Write the config's parameter and star files under out_dir (cached by
    name).  Returns paths and theta vectors."""
    os.makedirs(out_dir, exist_ok=True)
    cfg = config(idx)
    rng = cfg["rng"]
    files = []
    for w, (p, n) in enumerate(zip(cfg["problems"], cfg["stars"])):
        n = max(1, int(round(n * star_scale)))
        pf = os.path.join(out_dir, f"config{idx}_wedge{w}_params.txt")
        sf = os.path.join(out_dir, f"config{idx}_wedge{w}_stars{n}.txt")
        p.write(pf)
        stars_rng = np.random.Generator(np.random.PCG64(1000 + 17 * idx + w))
        if not os.path.exists(sf):
            write_stars(sf, sample_stars(p, n, stars_rng))
        files.append({"params": pf, "stars": sf, "theta": p.theta(), "problem": p, "n_stars": n})
    out = {"files": files}
    if "thetas" in cfg:
        out["thetas"] = cfg["thetas"]
    return out
