"""Host API mirroring the reference's C++ interface for the sinogram + circus path.

Names, argument meaning and error behaviour follow maleadt/tracetransform's
c++/src:

* ``TFunctionalWrapper.parse("0".."7")`` / ``PFunctionalWrapper.parse("1", "2",
  "3", "H<order>")`` -- the ``operator>>`` parsers (sinogram.cpp:34-65,
  circus.cpp:33-66); bad ids raise ``ValidationError``;
* ``pad(image)`` -- auxiliary.cpp:257-275;
* ``getSinograms(padded, angle_stepsize, tfunctionals)`` -- sinogram.cpp:67-178,
  returns one N x A float32 matrix per T-functional;
* ``getCircusFunctions(sinogram, pfunctionals)`` -- circus.cpp:104-177, returns
  one length-A vector per P-functional;
* ``zscore(vector)`` -- auxiliary.cpp:305-318;
* ``Transformer(image, basename, angle_stepsize, orthonormal).getTransform(
  tfunctionals, pfunctionals, write_data)`` -- transform.cpp:28-112, returning
  the A x (nT * nP) signature matrix (and writing ``<basename>.csv`` when
  ``write_data`` is true, as the reference does).

Matrices are numpy float32 arrays of shape (rows, cols); they are handed to
the engine in column-major (Eigen) order.  All compute runs on the GPU through
libtt_gb300.so; there is no CPU implementation here.
"""
from __future__ import annotations

import ctypes
import enum
import logging
import math
import re
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from . import _native
from ._native import PFunctionalC, check, fptr, iptr, lib

__all__ = [
    "TFunctional", "PFunctional", "TFunctionalWrapper", "PFunctionalWrapper", "ValidationError",
    "pad", "pad_geometry", "ortho_size", "angles_from_step", "getSinograms", "getCircusFunctions",
    "zscore", "Transformer", "writecsv", "Plan", "transform_batch", "rotate",
    "transform_extended",
]


class ValidationError(ValueError):
    """boost::program_options::validation_error(invalid_option_value)."""


class TFunctional(enum.IntEnum):
    Radon = 0
    T1 = 1
    T2 = 2
    T3 = 3
    T4 = 4
    T5 = 5
    T6 = 6
    T7 = 7


class PFunctional(enum.IntEnum):
    Hermite = 0
    P1 = 1
    P2 = 2
    P3 = 3


@dataclass
class TFunctionalWrapper:
    name: str
    functional: TFunctional

    @classmethod
    def parse(cls, text: str) -> "TFunctionalWrapper":
        """operator>>(istream, TFunctionalWrapper&) of c++/src/sinogram.cpp:34-65."""
        names = {"0": "Radon", "1": "T1", "2": "T2", "3": "T3", "4": "T4", "5": "T5",
                 "6": "T6", "7": "T7"}
        if text not in names:
            raise ValidationError(f"invalid T-functional {text!r}")
        return cls(names[text], TFunctional(int(text)))


@dataclass
class PFunctionalArguments:
    order: Optional[int] = None
    center: Optional[int] = None


@dataclass
class PFunctionalWrapper:
    name: str
    functional: PFunctional
    arguments: PFunctionalArguments = field(default_factory=PFunctionalArguments)

    @classmethod
    def parse(cls, text: str) -> "PFunctionalWrapper":
        """operator>>(istream, PFunctionalWrapper&) of c++/src/circus.cpp:33-66."""
        if text in ("1", "2", "3"):
            return cls("P" + text, PFunctional(int(text)))
        if text[:1] == "H":
            if len(text) < 2:
                raise ValidationError("Missing order parameter for Hermite P-functional")
            digits = text[1:]
            if not digits.isdigit():
                raise ValidationError("Unparseable order parameter for Hermite P-functional")
            return cls(text, PFunctional.Hermite, PFunctionalArguments(order=int(digits)))
        raise ValidationError(f"invalid P-functional {text!r}")


def _as_tfunctionals(tfunctionals) -> List[TFunctionalWrapper]:
    out = []
    for t in tfunctionals:
        if isinstance(t, TFunctionalWrapper):
            out.append(t)
        elif isinstance(t, str):
            out.append(TFunctionalWrapper.parse(t))
        else:
            out.append(TFunctionalWrapper.parse(str(int(t))))
    return out


def _as_pfunctionals(pfunctionals) -> List[PFunctionalWrapper]:
    out = []
    for p in pfunctionals:
        if isinstance(p, PFunctionalWrapper):
            out.append(p)
        else:
            out.append(PFunctionalWrapper.parse(str(p)))
    return out


class Plan:
    """Owns one tt_plan (device tables, staging buffers, stream) of a device."""

    def __init__(self, device: int = 0):
        h = ctypes.c_void_p()
        check(lib().tt_plan_create(ctypes.byref(h), int(device)))
        self.handle = h
        self.device = device

    def close(self):
        if self.handle:
            lib().tt_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def synchronize(self):
        check(lib().tt_plan_synchronize(self.handle))


def _handle(plan: Optional[Plan]):
    return plan.handle if plan is not None else None


def _colmajor(a) -> np.ndarray:
    """float32 copy of a 2-D matrix as a flat column-major buffer."""
    a = np.asarray(a, dtype=np.float32)
    if a.ndim != 2:
        raise ValueError("expected a 2-D matrix")
    return np.ascontiguousarray(a.ravel(order="F"))


def pad_geometry(rows: int, cols: int):
    """(N, row offset, col offset) of pad() (c++/src/auxiliary.cpp:257-275)."""
    n, ro, co = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    check(lib().tt_pad_geometry(int(rows), int(cols), ctypes.byref(n), ctypes.byref(ro),
                                ctypes.byref(co)))
    return n.value, ro.value, co.value


def pad(image) -> np.ndarray:
    """Zero-pad to the N x N frame that holds every rotation of the image."""
    image = np.asarray(image, dtype=np.float32)
    n, ro, co = pad_geometry(*image.shape)
    out = np.zeros((n, n), np.float32, order="F")
    out[ro:ro + image.shape[0], co:co + image.shape[1]] = image
    return out


def ortho_size(angle_stepsize: int) -> int:
    side = ctypes.c_int()
    check(lib().tt_ortho_size(int(angle_stepsize), ctypes.byref(side)))
    return side.value


def angles_from_step(angle_stepsize: int) -> np.ndarray:
    count = ctypes.c_int()
    check(lib().tt_angles_from_step(int(angle_stepsize), None, 0, ctypes.byref(count)))
    out = np.zeros(count.value, np.float32)
    check(lib().tt_angles_from_step(int(angle_stepsize), fptr(out), count.value, ctypes.byref(count)))
    return out


def getSinograms(padded, angle_stepsize: int, tfunctionals: Sequence,
                 plan: Optional[Plan] = None) -> List[np.ndarray]:
    """One N x A sinogram per T-functional (c++/src/sinogram.cpp:67-178)."""
    tfs = _as_tfunctionals(tfunctionals)
    padded = np.asarray(padded, dtype=np.float32)
    rows, cols = padded.shape
    if int(angle_stepsize) < 1:
        raise ValidationError("angle step must be >= 1")
    a = 360 // int(angle_stepsize)
    ids = np.array([int(t.functional) for t in tfs], np.int32)
    out = np.zeros(len(tfs) * rows * a, np.float32)
    check(lib().tt_sinograms(_handle(plan), fptr(_colmajor(padded)), rows, cols,
                             int(angle_stepsize), iptr(ids), len(ids), fptr(out)))
    stack = out.reshape(len(tfs), a, rows)
    return [np.asfortranarray(stack[t].T) for t in range(len(tfs))]


def _pf_array(pfs: List[PFunctionalWrapper]):
    arr = (PFunctionalC * max(len(pfs), 1))()
    for i, p in enumerate(pfs):
        arr[i].kind = int(p.functional)
        arr[i].order = -1 if p.arguments.order is None else int(p.arguments.order)
        arr[i].center = -1 if p.arguments.center is None else int(p.arguments.center)
    return arr


def getCircusFunctions(sinogram, pfunctionals: Sequence,
                       plan: Optional[Plan] = None) -> List[np.ndarray]:
    """One length-A circus function per P-functional (c++/src/circus.cpp:104-177)."""
    pfs = _as_pfunctionals(pfunctionals)
    sinogram = np.asarray(sinogram, dtype=np.float32)
    rows, cols = sinogram.shape
    for p in pfs:
        if p.functional == PFunctional.Hermite and (p.arguments.order is None or
                                                    p.arguments.center is None):
            raise ValidationError("Hermite P-functional needs an order and a center")
    out = np.zeros(len(pfs) * cols, np.float32)
    check(lib().tt_circus(_handle(plan), fptr(_colmajor(sinogram)), rows, cols, _pf_array(pfs),
                          len(pfs), fptr(out)))
    return [out[p * cols:(p + 1) * cols].copy() for p in range(len(pfs))]


def nearest_orthonormal_sinogram(sinogram, plan: Optional[Plan] = None):
    """(nos, new_center) of c++/src/circus.cpp:68-102 for one N x A sinogram:
    the columns aligned on their weighted medians and replaced by the polar
    factor U V^T (on the device: pivoted QR in double-float, one-sided
    Jacobi on R^T in float)."""
    sinogram = np.asarray(sinogram, dtype=np.float32)
    rows, cols = sinogram.shape
    out = np.zeros(2 * rows * cols, np.float32)
    m, c = ctypes.c_int32(), ctypes.c_int32()
    check(lib().tt_nos(_handle(plan), fptr(_colmajor(sinogram)), rows, cols, fptr(out),
                       ctypes.byref(m), ctypes.byref(c)))
    return out[: m.value * cols].reshape((m.value, cols), order="F"), c.value


def rotate(image, angle_degrees: float, plan: Optional[Plan] = None) -> np.ndarray:
    """rotate(image, ((cols-1)/2, (rows-1)/2), deg2rad(angle)) of
    c++/src/auxiliary.cpp:223-255, bit-identical to the reference."""
    image = np.asarray(image, dtype=np.float32)
    rows, cols = image.shape
    out = np.zeros(rows * cols, np.float32)
    check(lib().tt_rotate(_handle(plan), fptr(_colmajor(image)), rows, cols,
                          float(angle_degrees), fptr(out)))
    return out.reshape((rows, cols), order="F")


def resize(image, rows: int, cols: int, plan: Optional[Plan] = None) -> np.ndarray:
    """resize(input, rows, cols) of c++/src/auxiliary.cpp:198-221 (the
    orthonormal mode's stretch), bit-identical to the reference."""
    image = np.asarray(image, dtype=np.float32)
    if image.ndim != 2:
        raise ValueError("expected a 2-D matrix")
    out = np.zeros(int(rows) * int(cols), np.float32)
    check(lib().tt_resize(_handle(plan), fptr(_colmajor(image)), image.shape[0], image.shape[1],
                          int(rows), int(cols), fptr(out)))
    return out.reshape((int(rows), int(cols)), order="F")


def zscore(vector, plan: Optional[Plan] = None) -> np.ndarray:
    """(x - mean) / std with n - 1 (c++/src/auxiliary.cpp:305-318)."""
    x = np.ascontiguousarray(np.asarray(vector, dtype=np.float32).ravel())
    out = np.zeros_like(x)
    if x.size:
        check(lib().tt_zscore(_handle(plan), fptr(x), 1, x.size, fptr(out)))
    return out


def writecsv(filename: str, data) -> None:
    """writecsv of c++/src/auxiliary.cpp:130-146: ", "-separated rows, floats
    printed as a default C++ ostream prints them (6 significant digits)."""
    data = np.asarray(data)
    with open(filename, "w") as f:
        for row in data:
            f.write(", ".join(_ostream_float(float(v)) for v in row) + "\n")


def _ostream_float(v: float) -> str:
    if math.isnan(v):
        return "-nan" if math.copysign(1.0, v) < 0 else "nan"
    if math.isinf(v):
        return "inf" if v > 0 else "-inf"
    return "%g" % v


_log = logging.getLogger("tracetransform_gb300")
_PGM_WS = b" \t\n\r"


def _netpbm_skip(buf: bytes, pos: int) -> int:
    """Whitespace and comment skipping of readNetpbmValue
    (c++/src/auxiliary.cpp:26-37): a '#' at the start of a value runs to the
    end of its line."""
    n = len(buf)
    while pos < n:
        ch = buf[pos]
        if ch == 0x23:  # '#'
            nl = buf.find(b"\n", pos)
            pos = n if nl < 0 else nl + 1
        elif ch in _PGM_WS:
            pos += 1
        else:
            break
    return pos


def _netpbm_header_value(buf: bytes, pos: int, text: bool):
    """One header value as `stream >> value` reads it after the skip: a token
    up to the next space for the magic string, a run of digits for a size."""
    pos = _netpbm_skip(buf, pos)
    n = len(buf)
    while pos < n and buf[pos] in b" \t\n\r\x0b\x0c":
        pos += 1
    start = pos
    if text:
        while pos < n and buf[pos] not in b" \t\n\r\x0b\x0c":
            pos += 1
        if pos == start:
            raise RuntimeError("Error processing file")
        return buf[start:pos].decode("latin-1"), pos
    if pos < n and buf[pos] == 0x2B:  # '+'
        pos += 1
    digits = pos
    while pos < n and 0x30 <= buf[pos] <= 0x39:
        pos += 1
    if pos == digits:
        raise RuntimeError("Error processing file")
    return int(buf[digits:pos]), pos


def readnetpbm(filename: str) -> List[np.ndarray]:
    """readnetpbm of c++/src/auxiliary.cpp:47-99: an ASCII PGM (P2, one
    channel) or PPM (P3, three channels, interleaved per pixel) file as one
    int32 rows x cols matrix per channel.  Comments start with '#' and run to
    the end of the line.  A maxval other than 255 and data after the last
    pixel only log a warning, as in the reference; a missing or malformed
    value raises RuntimeError("Error processing file").  Pixel values are
    read as unsigned 32-bit integers and stored as int32 (so "-1" reads as
    -1, as the reference's unsigned read followed by its int store gives)."""
    try:
        with open(filename, "rb") as f:
            buf = f.read()
    except OSError as e:
        raise RuntimeError("could not open input file") from e
    magic, pos = _netpbm_header_value(buf, 0, True)
    if magic == "P2":
        channels = 1
    elif magic == "P3":
        channels = 3
    else:
        raise RuntimeError("Invalid Netpbm magic")
    cols, pos = _netpbm_header_value(buf, pos, False)
    rows, pos = _netpbm_header_value(buf, pos, False)
    maxval, pos = _netpbm_header_value(buf, pos, False)
    if maxval != 255:
        _log.warning("Pixels not properly clipped to [0,255]")
    count = rows * cols * channels
    # past the header a comment can only end a value, so blanking comments
    # out and splitting on whitespace reads the same values
    body = re.sub(rb"#[^\n]*\n?", b" ", buf[pos:])
    tokens = body.split()
    if len(tokens) < count:
        raise RuntimeError("Error processing file")
    if len(tokens) > count:
        _log.warning("Trailing data at end of image file")
    try:
        vals = np.array(tokens[:count]).astype(np.int64) if count else np.zeros(0, np.int64)
    except ValueError as e:
        raise RuntimeError("Error processing file") from e
    if count and (vals.max() > 0xFFFFFFFF or vals.min() < -0xFFFFFFFF):
        raise RuntimeError("Error processing file")
    vals = (vals & 0xFFFFFFFF).astype(np.uint32).view(np.int32)
    pix = vals.reshape(rows, cols, channels)
    return [np.asfortranarray(pix[:, :, c]) for c in range(channels)]


def writepgm(filename: str, data) -> None:
    """writepgm of c++/src/auxiliary.cpp:101-128: "P2", "cols rows", 255,
    then the values row by row, each followed by a space, or by a newline
    once the current line holds more than 66 characters."""
    data = np.asarray(data)
    if data.ndim != 2:
        raise ValueError("expected a 2-D matrix")
    out = ["P2\n%d %d\n255\n" % (data.shape[1], data.shape[0])]
    run = 0
    for v in data.astype(np.int64).ravel(order="C").tolist():
        t = str(v)
        run += len(t)
        if run > 66:
            out.append(t + "\n")
            run = 0
        else:
            out.append(t + " ")
            run += 1
    with open(filename, "w") as f:
        f.write("".join(out))


def gray2mat(data) -> np.ndarray:
    """gray2mat of c++/src/auxiliary.cpp:148-157: pixel / 255.0 in double,
    stored as float32 (column-major, as Eigen stores it)."""
    data = np.asarray(data)
    return np.asfortranarray((data.astype(np.float64) / 255.0).astype(np.float32))


def mat2gray(data) -> np.ndarray:
    """mat2gray of c++/src/auxiliary.cpp:159-178: scale by 255 / the largest
    value (at least 0) in double and truncate to int32.  Where that is not a
    finite int32 (an all-zero matrix divides 0 by 0) the value is INT32_MIN,
    the result the reference's x86-64 build gives for such a conversion."""
    data = np.asarray(data, dtype=np.float32)
    finite = data[~np.isnan(data)]
    maximum = np.float32(max(0.0, float(finite.max()))) if finite.size else np.float32(0.0)
    with np.errstate(divide="ignore", invalid="ignore"):
        scaled = data.astype(np.float64) * 255.0 / np.float64(maximum)
    ok = np.isfinite(scaled) & (scaled > -2147483649.0) & (scaled < 2147483648.0)
    out = np.full(data.shape, np.iinfo(np.int32).min, np.int32)
    out[ok] = np.trunc(scaled[ok]).astype(np.int32)
    return np.asfortranarray(out)


def transform_batch_flat(flat: np.ndarray, offsets, rows, cols, angle_stepsizes,
                         tfunctionals: Sequence, pfunctionals: Sequence,
                         plan: Optional[Plan] = None):
    """tt_transform_batch on images already packed column-major into one float32
    buffer at element offsets; returns flat (circus, signatures), image after
    image, n_t x n_p x A_i each."""
    tfs = _as_tfunctionals(tfunctionals)
    pfs = _as_pfunctionals(pfunctionals)
    flat = np.ascontiguousarray(flat, dtype=np.float32)
    offsets = np.ascontiguousarray(np.asarray(offsets, np.int64))
    r = np.ascontiguousarray(np.asarray(rows, np.int32))
    c = np.ascontiguousarray(np.asarray(cols, np.int32))
    steps = np.ascontiguousarray(np.asarray([int(s) for s in angle_stepsizes], np.int32))
    ids = np.array([int(t.functional) for t in tfs], np.int32)
    total = sum(len(ids) * len(pfs) * (360 // int(s)) for s in steps)
    circus = np.zeros(max(total, 1), np.float32)
    sig = np.zeros(max(total, 1), np.float32)
    check(lib().tt_transform_batch(
        _handle(plan), fptr(flat), offsets.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
        iptr(r), iptr(c), iptr(steps), len(r), iptr(ids), len(ids), _pf_array(pfs),
        len(pfs), fptr(circus), fptr(sig)))
    return circus[:total], sig[:total]


def transform_batch(images: Sequence, angle_stepsizes: Sequence[int], tfunctionals: Sequence,
                    pfunctionals: Sequence, plan: Optional[Plan] = None):
    """Transform many images of uneven sizes in one pass of the batched engine
    (tt_transform_batch): returns, per image, (circus, signatures) with circus
    of shape (nT, nP, A) and signatures the A x (nT * nP) matrix
    Transformer.getTransform returns.  P1-P3 only."""
    tfs = _as_tfunctionals(tfunctionals)
    pfs = _as_pfunctionals(pfunctionals)
    imgs = [np.asarray(im, dtype=np.float32) for im in images]
    if len(angle_stepsizes) != len(imgs):
        raise ValueError("one angle step per image")
    bufs = [_colmajor(im) for im in imgs]
    offsets = np.zeros(len(bufs), np.int64)
    if bufs:
        offsets[1:] = np.cumsum([b.size for b in bufs])[:-1]
    flat = np.concatenate(bufs) if bufs else np.zeros(1, np.float32)
    circus, sig = transform_batch_flat(flat, offsets, [im.shape[0] for im in imgs],
                                       [im.shape[1] for im in imgs], angle_stepsizes, tfs, pfs,
                                       plan)
    ids = [int(t.functional) for t in tfs]
    na = [360 // int(s) for s in angle_stepsizes]
    out, at = [], 0
    for a in na:
        k = len(ids) * len(pfs) * a
        c = circus[at:at + k].reshape(len(ids), len(pfs), a)
        s = sig[at:at + k].reshape(len(ids) * len(pfs), a).T
        out.append((c, s))
        at += k
    return out


def transform_extended(image, angles_deg, tfunctionals: Sequence, pfunctionals: Sequence,
                       hermite_orders: Sequence[int], plan: Optional[Plan] = None) -> dict:
    """tt_transform_extended: the regular circus functions (P1-P3) and the
    orthonormal Hermite circus of the same (unstretched) sinograms in one
    call, over an explicit angle list.  Returns circus / signatures of shape
    (nT, nP, A), hermite_circus / hermite_signatures (nT, nH, A) and the
    nT Hermite centers."""
    tfs = _as_tfunctionals(tfunctionals)
    pfs = _as_pfunctionals(pfunctionals)
    img = _colmajor(np.asarray(image, dtype=np.float32))
    rows, cols = np.shape(image)
    ang = np.ascontiguousarray(np.asarray(angles_deg, np.float32))
    ids = np.array([int(t.functional) for t in tfs], np.int32)
    orders = np.ascontiguousarray(np.asarray(hermite_orders, np.int32))
    nt, npf, nh, a = len(ids), len(pfs), len(orders), len(ang)
    out = {k: np.zeros((nt, m, a), np.float32) for k, m in
           (("circus", npf), ("signatures", npf), ("hermite_circus", nh),
            ("hermite_signatures", nh))}
    centers = np.zeros(max(nt, 1), np.int32)
    check(lib().tt_transform_extended(
        _handle(plan), fptr(img), rows, cols, fptr(ang), a, iptr(ids), nt, _pf_array(pfs), npf,
        iptr(orders), nh, fptr(out["circus"]), fptr(out["signatures"]),
        fptr(out["hermite_circus"]), fptr(out["hermite_signatures"]), iptr(centers)))
    out["centers"] = centers[:nt]
    return out


def _write_debug_sinograms(basename: str, tfs: List[TFunctionalWrapper], sinograms) -> None:
    for t, sino in zip(tfs, sinograms):
        writecsv(f"{basename}-{t.name}.csv", sino)
        writepgm(f"{basename}-{t.name}.pgm", mat2gray(sino))


class Transformer:
    """Transformer of c++/src/transform.hpp:24-38 on the GPU engine."""

    def __init__(self, image, basename: str, angle_stepsize: int, orthonormal: bool,
                 plan: Optional[Plan] = None):
        self._image = np.asarray(image, dtype=np.float32)
        self._basename = basename
        self._angle_stepsize = int(angle_stepsize)
        self._orthonormal = bool(orthonormal)
        self._plan = plan
        if self._angle_stepsize < 1:
            raise ValidationError("angle step must be >= 1")

    def getTransform(self, tfunctionals: Sequence, pfunctionals: Sequence,
                     write_data: bool = True, debug: bool = False) -> np.ndarray:
        """Sinograms -> [nearest orthonormal sinogram] -> circus -> z-score.

        Returns the A x (nT * nP) signature matrix; with write_data it is also
        written to <basename>.csv.  Hermite centers of pfunctionals are
        updated in place, as the reference does (transform.cpp:80-84).
        write_data with debug (the reference's debug log level) also writes
        each sinogram as <basename>-<T name>.csv and, through mat2gray, .pgm
        (transform.cpp:61-72)."""
        tfs = _as_tfunctionals(tfunctionals)
        pfs = _as_pfunctionals(pfunctionals)
        if write_data and debug:
            img = self._image
            if self._orthonormal:
                side = ortho_size(self._angle_stepsize)
                img = resize(img, side, side, self._plan)
            _write_debug_sinograms(self._basename, tfs,
                                   getSinograms(pad(img), self._angle_stepsize, tfs, self._plan))
        n_h = sum(1 for p in pfs if p.functional == PFunctional.Hermite)
        if n_h and n_h != len(pfs):
            raise ValidationError("Cannot mix regular and orthonormal P-functionals")
        if (n_h > 0) != self._orthonormal and pfs:
            raise ValidationError("orthonormal mode must match the P-functionals")
        rows, cols = self._image.shape
        a = 360 // self._angle_stepsize
        ids = np.array([int(t.functional) for t in tfs], np.int32)
        circus = np.zeros(len(tfs) * len(pfs) * a, np.float32)
        sig = np.zeros(len(tfs) * len(pfs) * a, np.float32)
        check(lib().tt_transform(_handle(self._plan), fptr(_colmajor(self._image)), rows, cols,
                                 self._angle_stepsize, iptr(ids), len(ids), _pf_array(pfs),
                                 len(pfs), fptr(circus), fptr(sig)))
        self.circus = circus.reshape(len(tfs), len(pfs), a)
        signatures = sig.reshape(len(tfs) * len(pfs), a).T
        if write_data and pfs:
            writecsv(self._basename + ".csv", signatures)
        return signatures
