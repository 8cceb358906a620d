"""ctypes binding of the CPU restatement (sph_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as the
checker and by bench.py's CPU-baseline leg.  Nothing in the product imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "sph_oracle.cpp"
BUILD_DIR = HERE / "_build"
LIB = BUILD_DIR / "liboracle.so"
GATHER, SCATTER = 0, 1

_DP = C.POINTER(C.c_double)
_lib = None


def build() -> Path:
    """g++ -O2 -ffp-contract=off -fopenmp (the expression order must not change)."""
    BUILD_DIR.mkdir(exist_ok=True)
    gxx = shutil.which("g++") or "g++"
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [gxx, "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           "-o", str(tmp), str(SRC)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
            build()
        L = C.CDLL(str(LIB))
        L.or_smooth_kernel.argtypes = [C.c_int, C.c_int, C.c_double, _DP, _DP, _DP]
        L.or_kernel_value.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double]
        L.or_kernel_value.restype = C.c_double
        L.or_kernel_gradient.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double]
        L.or_kernel_gradient.restype = C.c_double
        L.or_powi.argtypes = [C.c_double, C.c_int64]
        L.or_powi.restype = C.c_double
        L.or_neighbour.argtypes = [C.c_int, C.c_int, C.c_double, _DP, _DP, _DP, _DP, C.c_double, _DP, _DP, _DP, _DP,
                                   _DP]
        L.or_pair_list_bruteforce.argtypes = [C.c_int, C.c_int64, _DP, C.c_double, C.c_int64,
                                              C.POINTER(C.c_int64)]
        L.or_pair_list_bruteforce.restype = C.c_int64
        L.or_cell_keys.argtypes = [C.c_void_p, C.c_int64, _DP, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.or_neighbour_lists.argtypes = [C.c_void_p, C.c_int64, _DP, C.c_int64, C.POINTER(C.c_int64),
                                         C.POINTER(C.c_int64)]
        L.or_neighbour_lists.restype = C.c_int64
        L.or_neighbour_counts.argtypes = [C.c_void_p, C.c_int64, _DP, C.c_int64, _DP, C.POINTER(C.c_int64),
                                          C.POINTER(C.c_int64)]
        L.or_run_io.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.c_int64] + [_DP] * 7 + \
            [C.c_int64, _DP, _DP, _DP, C.POINTER(C.c_int32), C.c_void_p, C.c_int64] + [_DP] * 7 + \
            [C.POINTER(C.c_int64), C.c_int64] + [_DP] * 7 + [C.c_int64, C.c_int64, C.POINTER(C.c_int64)]
        L.or_run_io.restype = C.c_int
        L.or_probe.argtypes = [C.c_int, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int64, _DP, C.c_int64, _DP,
                               _DP, _DP, C.c_int, C.POINTER(_DP), C.c_double, _DP]
        L.or_probe.restype = C.c_int
        L.or_run.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_int64)] + [_DP] * 10 + \
            [C.c_int64] + [_DP] * 6 + [C.POINTER(C.c_int32), C.c_int64, C.c_int64]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(_DP)


def smooth_kernel(kind: int, dim: int, rc: float):
    h, s, k0 = C.c_double(), C.c_double(), C.c_double()
    assert lib().or_smooth_kernel(kind, dim, rc, C.byref(h), C.byref(s), C.byref(k0)) == 0
    return h.value, s.value, k0.value


def kernel_value(kind, dim, rc, r):
    return lib().or_kernel_value(kind, dim, rc, r)


def kernel_gradient(kind, dim, rc, r):
    return lib().or_kernel_gradient(kind, dim, rc, r)


def powi(x, n):
    return lib().or_powi(x, n)


def neighbour(kind, dim, rc, xi, xj, vi, vj, r):
    f = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    xi, xj, vi, vj = f(xi), f(xj), f(vi), f(vj)
    rv, vv, g = np.zeros(dim), np.zeros(dim), np.zeros(dim)
    W, dW = C.c_double(), C.c_double()
    assert lib().or_neighbour(kind, dim, rc, _p(xi), _p(xj), _p(vi), _p(vj), r, _p(rv), _p(vv), C.byref(W),
                              C.byref(dW), _p(g)) == 0
    return dict(r_vec=rv, v_vec=vv, W=W.value, dW=dW.value, grad=g)


def pair_list_bruteforce(x: np.ndarray, rc: float) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    n, dim = x.shape
    cnt = lib().or_pair_list_bruteforce(dim, n, _p(x), rc, 0, None)
    out = np.zeros((max(cnt, 1), 2), dtype=np.int64)
    lib().or_pair_list_bruteforce(dim, n, _p(x), rc, cnt, out.ctypes.data_as(C.POINTER(C.c_int64)))
    return out[:cnt]


def cell_keys(params, x: np.ndarray):
    x = np.ascontiguousarray(x, dtype=np.float64)
    keys = np.zeros(len(x), dtype=np.int64)
    nc = C.c_int64()
    assert lib().or_cell_keys(C.byref(params), len(x), _p(x), keys.ctypes.data_as(C.POINTER(C.c_int64)),
                              C.byref(nc)) == 0
    return keys, nc.value


def neighbour_lists(params, x: np.ndarray):
    """Full neighbour list of every particle (ids ascending) as (offsets[n+1], ids)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    n = len(x)
    offsets = np.zeros(n + 1, dtype=np.int64)
    P64 = C.POINTER(C.c_int64)
    total = lib().or_neighbour_lists(C.byref(params), n, _p(x), 0, offsets.ctypes.data_as(P64), None)
    assert total >= 0
    ids = np.zeros(max(total, 1), dtype=np.int64)
    assert lib().or_neighbour_lists(C.byref(params), n, _p(x), total, offsets.ctypes.data_as(P64),
                                    ids.ctypes.data_as(P64)) == total
    return offsets, ids[:total]


def neighbour_counts(params, x, wx):
    x = np.ascontiguousarray(x, dtype=np.float64)
    wx = np.ascontiguousarray(wx, dtype=np.float64) if wx is not None and len(wx) else np.zeros((0, x.shape[1]))
    a, b = C.c_int64(), C.c_int64()
    assert lib().or_neighbour_counts(C.byref(params), len(x), _p(x), len(wx), _p(wx), C.byref(a), C.byref(b)) == 0
    return a.value, b.value


def run(params, fluid: dict, walls: dict | None, first_step: int, nsteps: int, mode: int = GATHER,
        threads: int = 0) -> dict:
    """Run the restated eachStep! on copies of the fluid arrays.

    fluid: x, v (n x dim), rho, p, c, mass, gap [, t, kappa, cp]; walls: x, normal,
    gap, kind [, t, kappa, v].  Returns the updated fluid (deleted particles removed).
    """
    f = lambda a: np.ascontiguousarray(np.array(a, dtype=np.float64, copy=True))
    st = {k: f(fluid[k]) for k in ("x", "v", "rho", "p", "c", "mass", "gap")}
    n = len(st["rho"])
    for k in ("t", "kappa", "cp"):
        st[k] = f(fluid[k]) if k in fluid else np.zeros(n)
    n_io = C.c_int64(n)
    if walls is not None and len(walls["gap"]):
        w = {k: np.ascontiguousarray(walls[k], dtype=np.float64) for k in ("x", "normal", "gap")}
        nw = len(w["gap"])
        wt = np.ascontiguousarray(walls.get("t", np.zeros(nw)), dtype=np.float64)
        wk = np.ascontiguousarray(walls.get("kappa", np.zeros(nw)), dtype=np.float64)
        wv = np.ascontiguousarray(walls.get("v", np.zeros((nw, st["x"].shape[1]))), dtype=np.float64)
        kind = np.ascontiguousarray(walls["kind"], dtype=np.int32)
    else:
        nw = 0
        w = {"x": None, "normal": None, "gap": None}
        wt = wk = wv = None
        kind = np.zeros(1, dtype=np.int32)
    rc = lib().or_run(C.byref(params), mode, threads, C.byref(n_io), _p(st["x"]), _p(st["v"]), _p(st["rho"]),
                      _p(st["p"]), _p(st["c"]), _p(st["mass"]), _p(st["gap"]), _p(st["t"]), _p(st["kappa"]),
                      _p(st["cp"]), nw, _p(w["x"]), _p(w["normal"]), _p(w["gap"]), _p(wt), _p(wk), _p(wv),
                      kind.ctypes.data_as(C.POINTER(C.c_int32)), first_step, nsteps)
    if rc != 0:
        raise RuntimeError("oracle rejected the parameter block")
    m = n_io.value
    return {k: a[:m] for k, a in st.items()}


def probe(kind, dim, rc, points, x, mass, rho, fields, none_value=float("nan"), periodic_x=False, period=0.0):
    """kernelValueInterpolation restated (brute force, FP64): fields is a list of
    per-particle arrays; returns an array (len(fields), len(points))."""
    pts = np.ascontiguousarray(points, dtype=np.float64)
    xs = np.ascontiguousarray(x, dtype=np.float64)
    m = np.ascontiguousarray(mass, dtype=np.float64)
    r = np.ascontiguousarray(rho, dtype=np.float64)
    fs = [np.ascontiguousarray(f, dtype=np.float64) for f in fields]
    arr = (_DP * max(1, len(fs)))(*[_p(f) for f in fs])
    out = np.empty((len(fs), len(pts)))
    rc_ = lib().or_probe(kind, dim, rc, int(periodic_x), period, len(pts), _p(pts), len(xs), _p(xs), _p(m), _p(r),
                         len(fs), arr, none_value, _p(out))
    if rc_ != 0:
        raise ValueError("bad kernel")
    return out


def run_io(params, fluid: dict, walls: dict, rules, inlet: dict, outlet: dict, first_step: int, nsteps: int,
           extra: int = 0):
    """The inlet/outlet solve (gather mode): dicts of x, v (n, dim) and rho, p, c, mass,
    gap; walls: x, normal, gap, kind; rules: an SphBufferRules.  Returns (fluid, inlet,
    outlet) dicts in the reference's vector orders (fluid["id"]: ids, ascending).
    `extra` = room for fluid and outlet growth."""
    dim = params.dim
    keys = ("rho", "p", "c", "mass", "gap")

    def arrs(d, cap):
        n = len(d["rho"])
        out = {"x": np.zeros((cap, dim)), "v": np.zeros((cap, dim))}
        out["x"][:n] = d["x"]
        out["v"][:n] = d["v"]
        for k in keys:
            out[k] = np.zeros(cap)
            out[k][:n] = d[k]
        return n, out

    nf, F = arrs(fluid, len(fluid["rho"]) + extra)
    ni, I = arrs(inlet, len(inlet["rho"]))
    no, O = arrs(outlet, len(outlet["rho"]) + extra)
    wx = np.ascontiguousarray(walls["x"], dtype=np.float64)
    wn = np.ascontiguousarray(walls["normal"], dtype=np.float64)
    wg = np.ascontiguousarray(walls["gap"], dtype=np.float64)
    wk = np.ascontiguousarray(walls["kind"], dtype=np.int32)
    n_f, n_o = C.c_int64(nf), C.c_int64(no)
    ids = np.zeros(len(F["rho"]), dtype=np.int64)
    rc = lib().or_run_io(C.byref(params), C.byref(n_f), len(F["rho"]), *[_p(F[k]) for k in ("x", "v") + keys],
                         len(wg), _p(wx), _p(wn), _p(wg), wk.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(rules), ni,
                         *[_p(I[k]) for k in ("x", "v") + keys], C.byref(n_o), len(O["rho"]),
                         *[_p(O[k]) for k in ("x", "v") + keys], first_step, nsteps,
                         ids.ctypes.data_as(C.POINTER(C.c_int64)))
    if rc != 0:
        raise ValueError(f"or_run_io failed ({rc})")
    cut = lambda d, n: {k: a[:n].copy() for k, a in d.items()}
    fl = cut(F, n_f.value)
    fl["id"] = ids[: n_f.value].copy()
    return fl, cut(I, ni), cut(O, n_o.value)


def scene_arrays(scene):
    """Fluid and merged wall arrays of a scenes.Scene, in upload order."""
    fl = scene.fluid
    fluid = dict(x=fl.x_vec_, v=fl.v_vec_, rho=fl.rho_, p=fl.p_, c=fl.c_, mass=fl.mass_, gap=fl.gap_)
    if getattr(fl, "thermal", False):
        fluid.update(t=fl.t_, kappa=fl.kappa_, cp=fl.cp_)
    if not scene.walls:
        return fluid, None
    xs, ns, gs, ts, ks, vs, kinds = [], [], [], [], [], [], []
    for w in scene.walls:
        m = len(w)
        xs.append(w.x_vec_)
        ns.append(w.normal_vec_)
        gs.append(w.gap_)
        ts.append(getattr(w, "t_", np.zeros(m)))
        ks.append(getattr(w, "kappa_", np.zeros(m)))
        vs.append(getattr(w, "v_vec_", np.zeros((m, w.dim))))
        kinds.append(np.full(m, w.wall_kind, dtype=np.int32))
    cat = lambda a: np.ascontiguousarray(np.concatenate(a))
    walls = dict(x=cat(xs), normal=cat(ns), gap=cat(gs), t=cat(ts), kappa=cat(ks), v=cat(vs), kind=cat(kinds))
    return fluid, walls
