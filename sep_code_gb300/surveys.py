"""Seeded synthetic surveys (pure numpy; loads no native library).

``Survey`` holds what the reference reads from its SEP files (velocity model,
reflectivity image, source wavelet, data axes, acquisition).  The generators
build the synthetic stand-ins for the workloads the reference is run on (no
field data is available): the 128^3 anomaly model, the 512x512x400 layered
model and small parity cases.  ``ShotSetup`` is the set of C ABI inputs one
shot needs; ``extract_sub`` and ``laplac_forward`` are the two image
preparations ``rtm_zero_op::forward`` applies before the Born call
(Born/rtm_zero_op_3d.cpp:147-153).

Both arms of the benchmark and the oracle side of the tests build their
inputs from this module, so nothing here may import the product library.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

FAT = 4


@dataclass
class Survey:
    vel: np.ndarray                 # model velocity (m/s), float32[m3, m2, m1]
    spacing: tuple                  # (d1, d2, d3) metres
    refl: np.ndarray                # reflectivity / image on the model grid
    wavelet: np.ndarray             # source wavelet (before the time derivative)
    dtw: float                      # wavelet sampling
    data_nt: int                    # samples per recorded trace
    data_dt: float
    rec: tuple                      # (rnx, rny, ro2, rd2, ro3, rd3)
    rec_depth: float = 0.0
    shots: list = field(default_factory=list)   # [(sx, sy, sz)] metres
    nbound: int = 20
    bc_a: float = 50.0
    bc_b: float = 0.0005
    name: str = "survey"


@dataclass
class ShotSetup:
    """C ABI inputs for one shot, as rtm_zero_op prepares them."""
    n: tuple                # padded (n1, n2, n3)
    o: tuple                # padded origins
    d: tuple
    dt: float               # propagation step
    nt: int                 # propagation steps
    jts: int
    jtd: int
    sinc_s: np.ndarray
    sinc_d: np.ndarray
    src_locs: np.ndarray
    src_vals: np.ndarray    # [9][nt_big]
    nt_big: int
    vel2dt2: np.ndarray     # random-boundary v^2 dt^2, [n3, n2, n1]
    rec_locs: np.ndarray
    rnx: int
    rny: int
    img_lap: np.ndarray | None = None   # laplac(extract_sub(image)) on the padded grid


def ricker(f0: float, dt: float, nt: int, t0: float | None = None) -> np.ndarray:
    t0 = 1.2 / f0 if t0 is None else t0
    t = np.arange(nt) * dt - t0
    a = (np.pi * f0 * t) ** 2
    return ((1 - 2 * a) * np.exp(-a)).astype(np.float32)


def anomaly_survey(n: int = 128, nt: int = 1000, seed: int = 20261204) -> Survey:
    """128^3, dx=10 m, dt=1 ms: v(z)=1500+0.6 z plus a +300 m/s Gaussian
    (sigma 150 m) at the centre; 5 flat horizons with N(0,0.05) amplitudes and
    ~2% sparse spikes; 15 Hz Ricker at the surface centre; receivers at every
    surface node; 20-cell random boundary."""
    rng = np.random.default_rng(seed)
    d = 10.0
    z = np.arange(n) * d
    x = np.arange(n) * d
    Z, Y, X = np.meshgrid(z, x, x, indexing="ij")
    c = (n - 1) * d / 2
    vel = 1500.0 + 0.6 * Z + 300.0 * np.exp(-((X - c) ** 2 + (Y - c) ** 2 + (Z - c) ** 2) / (2 * 150.0 ** 2))
    refl = np.zeros((n, n, n), np.float32)
    for iz in np.sort(rng.choice(np.arange(n // 8, n - n // 8), 5, replace=False)):
        refl[iz] += rng.normal(0, 0.05)
    spikes = rng.random((n, n, n)) < 0.02
    refl[spikes] += rng.normal(0, 0.05, spikes.sum()).astype(np.float32)
    w = ricker(15.0, 0.001, nt)
    return Survey(vel=vel.astype(np.float32), spacing=(d, d, d), refl=refl, wavelet=w, dtw=0.001,
                  data_nt=nt, data_dt=0.001, rec=(n, n, 0.0, d, 0.0, d),
                  shots=[(c, c, 0.0)], nbound=20, name=f"anomaly_{n}")


def layered_survey(n1: int = 512, n2: int = 512, n3: int = 400, nt: int = 4000,
                   seed: int = 20261205) -> Survey:
    """512x512x400, dx=12.5 m, dt=1 ms: seeded layered 1500-4500 m/s velocity
    with 8 random-depth dipping interfaces and smooth lateral perturbations;
    20 Hz Ricker; 512x512 surface receivers."""
    rng = np.random.default_rng(seed)
    d = 12.5
    x = (np.arange(n1) * d).astype(np.float32)
    y = (np.arange(n2) * d).astype(np.float32)
    zz = (np.arange(n3) * d).astype(np.float32)
    depth = n3 * d
    ifaces = np.sort(rng.uniform(0.05, 0.95, 8)) * depth
    dips = rng.uniform(-0.08, 0.08, (8, 2))
    vlay = np.linspace(1500.0, 4500.0, 9)
    Y, X = np.meshgrid(y, x, indexing="ij")
    pert = (60.0 * np.sin(2 * np.pi * X / (n1 * d) * rng.uniform(1, 3)) *
            np.cos(2 * np.pi * Y / (n2 * d) * rng.uniform(1, 3))).astype(np.float32)
    vel = np.empty((n3, n2, n1), np.float32)
    surf = np.stack([ifaces[k] + dips[k, 0] * (X - X.mean()) + dips[k, 1] * (Y - Y.mean())
                     for k in range(8)])
    for iz in range(n3):
        layer = (zz[iz] > surf).sum(axis=0)
        vel[iz] = vlay[layer] + pert
    vel = np.clip(vel, 1500.0, 4500.0)
    refl = np.zeros_like(vel)
    dv = np.diff(vel, axis=0)
    refl[1:] = np.where(np.abs(dv) > 50, dv / (2 * vel[1:]), 0.0)
    w = ricker(20.0, 0.001, nt)
    return Survey(vel=vel, spacing=(d, d, d), refl=refl.astype(np.float32), wavelet=w, dtw=0.001,
                  data_nt=nt, data_dt=0.001, rec=(n1, n2, 0.0, d, 0.0, d),
                  shots=[((n1 - 1) * d / 2, (n2 - 1) * d / 2, 0.0)], nbound=20,
                  name=f"layered_{n1}x{n2}x{n3}")


def small_survey(m1=24, m2=20, m3=28, nt=60, d=10.0, nbound=4, seed=7, rnx=None, rny=None,
                 dtw=None, data_dt=0.002) -> Survey:
    """A few-second case for parity tests: smooth model with an anomaly,
    random reflectivity, 25 Hz Ricker, partial receiver spread."""
    rng = np.random.default_rng(seed)
    z = np.arange(m3)[:, None, None] * d
    vel = (1800.0 + 2.0 * z + 100.0 * rng.standard_normal((m3, m2, m1)).cumsum(0) / m3)
    vel = np.broadcast_to(vel, (m3, m2, m1)).astype(np.float32).copy()
    refl = (rng.standard_normal((m3, m2, m1)) * (rng.random((m3, m2, m1)) < 0.1)).astype(np.float32)
    dtw = data_dt if dtw is None else dtw
    w = ricker(25.0, dtw, nt)
    rnx = m1 - 4 if rnx is None else rnx
    rny = m2 - 4 if rny is None else rny
    return Survey(vel=vel, spacing=(d, d, d), refl=refl, wavelet=w, dtw=dtw, data_nt=nt,
                  data_dt=data_dt, rec=(rnx, rny, 2 * d, d, 2 * d, d), rec_depth=0.0,
                  shots=[(m1 * d / 2, m2 * d / 2, 0.0)], nbound=nbound, bc_a=20.0, bc_b=0.002,
                  name="small")


def padded_origins(s: Survey, fat: int = FAT):
    """source_func::create_domain: o = -d * (nbound + fat) in float; d as float."""
    nb = s.nbound + fat
    d = tuple(float(np.float32(v)) for v in s.spacing)
    o = tuple(float(-np.float32(dd) * np.float32(nb)) for dd in d)
    return o, d


def extract_sub(s: Survey, n, o):
    """image_rtm_3d::extract_sub (Born/image_rtm_3d.cpp:52-90) with a unit mute."""
    m3, m2, m1 = s.refl.shape
    img = np.zeros((n[2], n[1], n[0]), np.float32)
    # f = (int)((o_in - o_model)/d_model): output index i reads model index i + f
    f = [int(np.float32(o[k]) / np.float32(s.spacing[k])) for k in range(3)]
    i1 = np.arange(n[0]) + f[0]
    i2 = np.arange(n[1]) + f[1]
    i3 = np.arange(n[2]) + f[2]
    v1 = (i1 >= 0) & (i1 < m1)
    v2 = (i2 >= 0) & (i2 < m2)
    v3 = (i3 >= 0) & (i3 < m3)
    sub = s.refl[np.ix_(i3[v3], i2[v2], i1[v1])]
    img[np.ix_(np.where(v3)[0], np.where(v2)[0], np.where(v1)[0])] = sub
    return img


def laplac_forward(m):
    """laplac::forward (Born/laplac_3d.cpp:46-96): a first difference along z."""
    d = np.zeros_like(m)
    d[1:] += m[:-1]
    d[:-1] -= m[:-1]
    return d
