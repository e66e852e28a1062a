"""ctypes front end to the CPU oracle (test infrastructure only).

Two checkers live here:

* ``liboracle.so`` -- the C restatement of the reference float path
  (oracle/tt_oracle.c), usable on any machine after ``make -C oracle``;
* ``_ref/ttref`` -- the reference's own c++/ sources compiled against the
  stand-in headers in oracle/shim/ (``make -C oracle ref``); only where a
  checkout of the reference exists.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this module.  The product package never does.

Array conventions: matrices are numpy arrays of shape (rows, cols) in Fortran
order (the reference's Eigen storage); a stack of sinograms is (nT, N, A).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_BIN = os.path.join(HERE, "_ref", "ttref")
REF_OMP_BIN = os.path.join(HERE, "_ref", "ttref_omp")

T_IDS = {"0": 0, "1": 1, "2": 2, "3": 3, "4": 4, "5": 5, "6": 6, "7": 7}
HERMITE, P1, P2, P3 = 0, 1, 2, 3

_lib = None
_F = ctypes.POINTER(ctypes.c_float)
_I = ctypes.POINTER(ctypes.c_int)


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        l = ctypes.CDLL(LIB_PATH)
        l.tto_deg2rad.restype = ctypes.c_float
        l.tto_deg2rad.argtypes = [ctypes.c_float]
        l.tto_rotation.argtypes = [ctypes.c_float, _F, _F]
        l.tto_pad_geometry.argtypes = [ctypes.c_int, ctypes.c_int, _I, _I, _I]
        l.tto_pad.argtypes = [_F, ctypes.c_int, ctypes.c_int, _F]
        l.tto_resize.argtypes = [_F, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _F]
        l.tto_rotate.argtypes = [_F, ctypes.c_int, ctypes.c_int, ctypes.c_float, _F]
        l.tto_zscore.argtypes = [_F, ctypes.c_int, _F]
        l.tto_find_weighted_median.argtypes = [_F, ctypes.c_int]
        l.tto_find_weighted_median.restype = ctypes.c_int
        for name in ("tto_t_radon", "tto_t1", "tto_t2", "tto_t6", "tto_t7",
                     "tto_p1", "tto_p2", "tto_p3"):
            fn = getattr(l, name)
            fn.argtypes = [_F, ctypes.c_int]
            fn.restype = ctypes.c_float
        l.tto_t345_prepare.argtypes = [ctypes.c_int, ctypes.c_int, _F, _F]
        l.tto_t345.argtypes = [_F, ctypes.c_int, _F, _F]
        l.tto_t345.restype = ctypes.c_float
        l.tto_t_at.argtypes = [ctypes.c_int, _F, ctypes.c_int, ctypes.c_int]
        l.tto_t_at.restype = ctypes.c_float
        l.tto_hermite_function.argtypes = [ctypes.c_uint, ctypes.c_float]
        l.tto_hermite_function.restype = ctypes.c_float
        l.tto_p_hermite.argtypes = [_F, ctypes.c_int, ctypes.c_uint, ctypes.c_int]
        l.tto_p_hermite.restype = ctypes.c_float
        l.tto_dft_r2c.argtypes = [_F, ctypes.c_int, _F, _F]
        l.tto_sinograms.argtypes = [_F, ctypes.c_int, _F, ctypes.c_int, _I, ctypes.c_int,
                                    _F, _I, ctypes.c_int]
        l.tto_circus.argtypes = [_F, ctypes.c_int, ctypes.c_int, _I, _I, _I, ctypes.c_int,
                                 _F, ctypes.c_int]
        l.tto_nos.argtypes = [_F, ctypes.c_int, ctypes.c_int, _F, _I, _I]
        l.tto_nos.restype = ctypes.c_int
        _lib = l
    return _lib


def _fp(a: np.ndarray):
    return a.ctypes.data_as(_F)


def _ip(a: np.ndarray):
    return a.ctypes.data_as(_I)


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32).ravel(order="F"))


def pad_geometry(rows: int, cols: int):
    n, ro, co = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    lib().tto_pad_geometry(rows, cols, ctypes.byref(n), ctypes.byref(ro), ctypes.byref(co))
    return n.value, ro.value, co.value


def pad(image: np.ndarray) -> np.ndarray:
    rows, cols = image.shape
    n, _, _ = pad_geometry(rows, cols)
    out = np.zeros(n * n, np.float32)
    lib().tto_pad(_fp(_f32(image)), rows, cols, _fp(out))
    return out.reshape((n, n), order="F")


def resize(image: np.ndarray, rows: int, cols: int) -> np.ndarray:
    out = np.zeros(rows * cols, np.float32)
    lib().tto_resize(_fp(_f32(image)), image.shape[0], image.shape[1], rows, cols, _fp(out))
    return out.reshape((rows, cols), order="F")


def rotate(image: np.ndarray, angle_deg: float) -> np.ndarray:
    rows, cols = image.shape
    out = np.zeros(rows * cols, np.float32)
    l = lib()
    l.tto_rotate(_fp(_f32(image)), rows, cols, l.tto_deg2rad(ctypes.c_float(angle_deg)), _fp(out))
    return out.reshape((rows, cols), order="F")


def t_at(f: int, x: np.ndarray, median: int) -> float:
    """T-functional f of column x with the weighted median held at row
    `median` (the reference's arithmetic, c++/src/functionals.cpp:95-276)."""
    x = np.ascontiguousarray(x, np.float32)
    return float(lib().tto_t_at(int(f), _fp(x), x.size, int(median)))


def t345_tables(which: int, n: int):
    """T3/T4/T5 kernels re, im (n floats each) as the reference rounds them
    (c++/src/functionals.cpp:136-198)."""
    re, im = np.zeros(n, np.float32), np.zeros(n, np.float32)
    lib().tto_t345_prepare(int(which), int(n), _fp(re), _fp(im))
    return re, im


def weighted_median(x: np.ndarray) -> int:
    """findWeightedMedian (c++/src/functionals.cpp:21-30)."""
    x = np.ascontiguousarray(x, np.float32)
    return int(lib().tto_find_weighted_median(_fp(x), x.size))


def angles_for_step(step) -> np.ndarray:
    """Angles in degrees: a_step * step for a_step in [0, floor(360/step))
    (c++/src/sinogram.cpp:77, 112); integer steps are exactly the reference's."""
    if float(step) == int(step):
        k = 360 // int(step)
    else:
        k = int(np.floor(360.0 / float(step)))
    return (np.arange(k, dtype=np.float64) * float(step)).astype(np.float32)


def sinograms(padded: np.ndarray, angles_deg, tfuncs, threads: int = 0,
              with_medians: bool = False):
    n = padded.shape[0]
    ang = np.ascontiguousarray(np.asarray(angles_deg, np.float32))
    tf = np.ascontiguousarray(np.asarray(tfuncs, np.int32))
    out = np.zeros(len(tf) * n * len(ang), np.float32)
    med = np.zeros(len(tf) * n * len(ang), np.int32) if with_medians else None
    lib().tto_sinograms(_fp(_f32(padded)), n, _fp(ang), len(ang), _ip(tf), len(tf), _fp(out),
                        _ip(med) if med is not None else None, threads)
    sino = out.reshape(len(tf), len(ang), n).transpose(0, 2, 1)
    if with_medians:
        return sino, med.reshape(len(tf), len(ang), n).transpose(0, 2, 1)
    return sino


def circus(sino: np.ndarray, pfuncs, threads: int = 0) -> np.ndarray:
    """pfuncs: list of (kind, order, center) tuples; returns (nP, cols)."""
    rows, cols = sino.shape
    kinds = np.array([p[0] for p in pfuncs], np.int32)
    orders = np.array([p[1] for p in pfuncs], np.int32)
    centers = np.array([p[2] for p in pfuncs], np.int32)
    out = np.zeros(len(pfuncs) * cols, np.float32)
    lib().tto_circus(_fp(_f32(sino)), rows, cols, _ip(kinds), _ip(orders), _ip(centers),
                     len(pfuncs), _fp(out), threads)
    return out.reshape(len(pfuncs), cols)


def zscore(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, np.float32)
    out = np.zeros_like(x)
    lib().tto_zscore(_fp(x), x.size, _fp(out))
    return out


def nos(sino: np.ndarray):
    rows, cols = sino.shape
    out = np.zeros(2 * rows * cols, np.float32)
    m, c = ctypes.c_int(), ctypes.c_int()
    rc = lib().tto_nos(_fp(_f32(sino)), rows, cols, _fp(out), ctypes.byref(m), ctypes.byref(c))
    if rc != 0:
        raise ValueError("nearest orthonormal sinogram needs rows + padding >= cols")
    return out[: m.value * cols].reshape((m.value, cols), order="F"), c.value


def ortho_size(step: int) -> int:
    """Side the orthonormal mode stretches images to (c++/src/transform.cpp:35-41)."""
    ndiag = int(np.ceil(360.0 / step))
    return int(np.ceil(ndiag / np.sqrt(2)))


def transform(image: np.ndarray, step: int, tfuncs, pfuncs, threads: int = 0):
    """Transformer(image, step, ortho) + getTransform (c++/src/transform.cpp:28-112).

    pfuncs: list of (kind, order) with kind in {HERMITE, P1, P2, P3}.
    Returns dict(padded, sino (nT,N,A), circus (nT,nP,A), sig (A, nT*nP),
    and, in orthonormal mode, nos (list) and centers (list))."""
    kinds = [p[0] for p in pfuncs]
    n_h = sum(1 for k in kinds if k == HERMITE)
    if n_h and n_h != len(kinds):
        raise ValueError("Cannot mix regular and orthonormal P-functionals")
    ortho = n_h > 0
    img = image
    if ortho:
        s = ortho_size(step)
        img = resize(img, s, s)
    padded = pad(img)
    ang = angles_for_step(step)
    sino = sinograms(padded, ang, tfuncs, threads)
    a = len(ang)
    circ = np.zeros((len(tfuncs), len(pfuncs), a), np.float32)
    sig = np.zeros((a, len(tfuncs) * len(pfuncs)), np.float32, order="F")
    res = {"padded": padded, "sino": sino, "circus": circ, "sig": sig}
    if ortho:
        res["nos"], res["centers"] = [], []
    for t in range(len(tfuncs)):
        s_t = sino[t]
        centers = [0] * len(pfuncs)
        if ortho:
            s_t, c = nos(s_t)
            res["nos"].append(s_t)
            res["centers"].append(c)
            centers = [c] * len(pfuncs)
        if pfuncs:
            cf = circus(s_t, [(k, o, centers[i]) for i, (k, o) in enumerate(pfuncs)], threads)
            circ[t] = cf
            for p in range(len(pfuncs)):
                sig[:, t * len(pfuncs) + p] = zscore(cf[p])
    return res


# ---------------------------------------------------------------------------
# the reference's own sources, built against the stand-ins (this machine only)
# ---------------------------------------------------------------------------

def ref_available() -> bool:
    return os.path.exists(REF_BIN)


def _pspec(pfuncs) -> str:
    if not pfuncs:
        return "-"
    return ",".join(f"H{o}" if k == HERMITE else str(k) for k, o in pfuncs)


def ref_transform(image: np.ndarray, step: int, tfuncs, pfuncs):
    rows, cols = image.shape
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "img.f32")
        _f32(image).tofile(src)
        prefix = os.path.join(d, "out")
        subprocess.run([REF_BIN, "transform", src, str(rows), str(cols), str(step),
                        ",".join(str(t) for t in tfuncs), _pspec(pfuncs), prefix], check=True)
        meta = {}
        centers = []
        for line in open(prefix + ".meta"):
            k, *v = line.split()
            if k == "center":
                centers.append((int(v[0]), int(v[1])))
            else:
                meta[k] = int(v[0])
        n, a = meta["n"], meta["angles"]
        nt, npf = len(tfuncs), len(pfuncs)
        res = {
            "padded": np.fromfile(prefix + ".padded.f32", np.float32).reshape((n, n), order="F"),
            "sino": np.fromfile(prefix + ".sino.f32", np.float32).reshape(nt, a, n).transpose(0, 2, 1),
            "circus": np.fromfile(prefix + ".circus.f32", np.float32).reshape(nt, npf, a),
            "sig": np.fromfile(prefix + ".sig.f32", np.float32).reshape((a, nt * npf), order="F"),
        }
        if meta.get("ortho"):
            raw = np.fromfile(prefix + ".nos.f32", np.float32)
            res["nos"], res["centers"], off = [], [], 0
            for c, m in centers:
                res["nos"].append(raw[off: off + m * a].reshape((m, a), order="F"))
                res["centers"].append(c)
                off += m * a
        return res


def ref_rotate(image: np.ndarray, angle_deg: float) -> np.ndarray:
    rows, cols = image.shape
    with tempfile.TemporaryDirectory() as d:
        src, dst = os.path.join(d, "img.f32"), os.path.join(d, "rot.f32")
        _f32(image).tofile(src)
        subprocess.run([REF_BIN, "rotate", src, str(rows), str(cols), repr(float(angle_deg)), dst],
                       check=True)
        return np.fromfile(dst, np.float32).reshape((rows, cols), order="F")


def ref_resize(image: np.ndarray, rows: int, cols: int) -> np.ndarray:
    """resize() run by the reference's own sources."""
    in_rows, in_cols = image.shape
    with tempfile.TemporaryDirectory() as d:
        src, dst = os.path.join(d, "img.f32"), os.path.join(d, "out.f32")
        _f32(image).tofile(src)
        subprocess.run([REF_BIN, "resize", src, str(in_rows), str(in_cols), str(rows), str(cols),
                        dst], check=True)
        return np.fromfile(dst, np.float32).reshape((rows, cols), order="F")


def ref_netpbm(text: bytes) -> dict:
    """readnetpbm / gray2mat / writepgm run by the reference's own sources on
    the file contents `text`: {"pixels": [...], "gray": [...], "pgm": [...]}
    per channel, or {"error": message} when the reader throws."""
    with tempfile.TemporaryDirectory() as d:
        src, prefix = os.path.join(d, "in.pgm"), os.path.join(d, "out")
        with open(src, "wb") as f:
            f.write(text)
        r = subprocess.run([REF_BIN, "netpbm", src, prefix], capture_output=True)
        if r.returncode != 0:
            return {"error": r.stderr.decode().strip()}
        meta = open(prefix + ".meta").read().split("\n")
        out = {"pixels": [], "gray": [], "pgm": [], "log": r.stderr.decode()}
        for i, line in enumerate(l for l in meta[1:] if l.startswith("shape")):
            rows, cols = (int(v) for v in line.split()[1:])
            base = f"{prefix}.c{i}"
            out["pixels"].append(np.fromfile(base + ".i32", np.int32).reshape((rows, cols), order="F"))
            out["gray"].append(np.fromfile(base + ".gray.f32", np.float32).reshape((rows, cols), order="F"))
            out["pgm"].append(open(base + ".pgm", "rb").read())
        return out


def ref_mat2gray(image: np.ndarray):
    """mat2gray run by the reference's own sources: (int32 matrix, writepgm
    text of it)."""
    rows, cols = image.shape
    with tempfile.TemporaryDirectory() as d:
        src, prefix = os.path.join(d, "img.f32"), os.path.join(d, "out")
        _f32(image).tofile(src)
        subprocess.run([REF_BIN, "mat2gray", src, str(rows), str(cols), prefix], check=True)
        gray = np.fromfile(prefix + ".i32", np.int32).reshape((rows, cols), order="F")
        return gray, open(prefix + ".pgm", "rb").read()
