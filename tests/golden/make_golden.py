"""Regenerate the golden fixtures in this folder from the reference itself.

Runs maleadt/tracetransform's own c++/ sources, compiled unmodified against
the stand-in headers in oracle/shim/ (``make -C oracle ref``; needs a checkout
of the reference, by default /root/reference), on seeded synthetic images and
stores inputs and outputs as compressed .npz files:

    python tests/golden/make_golden.py        # transform / rotate fixtures
    python tests/golden/make_golden.py io     # resize and image I/O fixtures

The fixtures pin the C restatement in oracle/ (tests/test_oracle_golden.py)
on machines without the reference checkout.
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from tracetransform_gb300.synthetic import blob_image  # noqa: E402

P123 = [(O.P1, 0), (O.P2, 0), (O.P3, 0)]
ALL_T = [0, 1, 2, 3, 4, 5, 6, 7]

# name: (image factory, angle step, T list, P list)
CASES = {
    "blob32_step4": (lambda: blob_image(32, 32, 5, (3, 10), (40, 200), 11), 4, ALL_T, P123),
    "blob20x13_step7": (lambda: blob_image(20, 13, 5, (3, 10), (40, 200), 12), 7, ALL_T, P123),
    "blob16x30_step3": (lambda: blob_image(16, 30, 4, (2, 8), (40, 200), 15), 3, ALL_T, P123),
    "blob48_ortho_step4": (lambda: blob_image(48, 48, 5, (3, 10), (40, 200), 13), 4, [0, 1, 2, 5],
                           [(O.HERMITE, 1), (O.HERMITE, 2), (O.HERMITE, 3), (O.HERMITE, 5)]),
    "zeros12_step5": (lambda: np.zeros((12, 12), np.float32, order="F"), 5, ALL_T, [(O.P1, 0), (O.P3, 0)]),
    "const9_step6": (lambda: np.full((9, 9), 0.5, np.float32, order="F"), 6, ALL_T, P123),
    "tiny3_step9": (lambda: blob_image(3, 3, 1, (1, 2), (40, 200), 16), 9, ALL_T, P123),
}

ROT_ANGLES = [0.0, 1.0, 17.0, 45.0, 90.0, 133.0, 180.0, 271.0, 359.0]


def impulse9():
    img = np.zeros((9, 9), np.float32, order="F")
    img[4, 4] = 1.0
    img[2, 6] = 200 / 255.0
    img[6, 1] = 77 / 255.0
    return img


def main():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    for name, (factory, step, tf, pf) in CASES.items():
        img = factory()
        res = O.ref_transform(img, step, tf, pf)
        out = {"image": img, "step": np.int32(step), "tfuncs": np.array(tf, np.int32),
               "pkinds": np.array([p[0] for p in pf], np.int32),
               "porders": np.array([p[1] for p in pf], np.int32)}
        for k in ("padded", "sino", "circus", "sig"):
            out[k] = res[k]
        if "nos" in res:
            out["centers"] = np.array(res["centers"], np.int32)
            for t, m in enumerate(res["nos"]):
                out[f"nos{t}"] = m
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, {k: getattr(v, "shape", v) for k, v in out.items()})
    img = impulse9()
    rots = np.stack([O.ref_rotate(img, a) for a in ROT_ANGLES])
    np.savez_compressed(os.path.join(HERE, "rotate9.npz"), image=img,
                        angles=np.array(ROT_ANGLES, np.float32), rotated=rots)
    print("rotate9", rots.shape)


# resize(): (input rows, cols, seed) -> output rows, cols.  Only cases whose
# samples all stay inside the image: the reference reads outside the input
# for the others (an assert in its debug build), e.g. a non-square image
# stretched to a square, or an up-scale by about 3x or more.
RESIZE_CASES = [((48, 48, 21), (64, 64)), ((64, 64, 22), (46, 46)), ((20, 13, 23), (26, 17)),
                ((13, 20, 24), (10, 15)), ((5, 5, 25), (3, 3)), ((3, 3, 26), (5, 5)),
                ((7, 7, 27), (2, 2)), ((30, 30, 28), (1, 5)), ((1024, 1024, None), (128, 128))]


def _resize_input(rows, cols, seed):
    if seed is not None:
        return np.asfortranarray(np.random.default_rng(seed).random((rows, cols)).astype(np.float32))
    # large case: a gray-level pattern (compresses well), as gray2mat scales it
    r, c = np.meshgrid(np.arange(rows), np.arange(cols), indexing="ij")
    return np.asfortranarray((((r * 37 + c * 11) % 256) / 255.0).astype(np.float32))


def _pgm_cases():
    """ASCII Netpbm inputs: layouts, comments, warnings and errors."""
    rng = np.random.default_rng(31)
    big = rng.integers(0, 256, size=(37, 53))
    big_text = "P2\n53 37\n255\n" + "\n".join(" ".join(str(v) for v in row) for row in big) + "\n"
    ppm = rng.integers(0, 256, size=(6, 5, 3))
    ppm_text = "P3\n# a colour image\n5 6\n255\n" + "\n".join(
        "  ".join(" ".join(str(v) for v in px) for px in row) for row in ppm) + "\n"
    return [
        big_text.encode(),
        ppm_text.encode(),
        b"P2\r\n# created by hand\r\n4 3\r\n# maxval next\r\n255\r\n"
        b"0 1 2 3\r\n4 5 6 7#end of row\r\n8 9 10 11\r\n",
        b"P2 3 2 65535 0 300 65535 7 8 9",            # maxval warning, values > 255
        b"P2\n2 2\n255\n1 2\n3 4\n5 6\n",             # trailing data warning
        b"P2\n2 2\n255\n1 -1\n+3 4294967295\n",       # unsigned read, int store
        b"P2\t2\t1\t255\t\t9\t10",
        b"P2\n0 0\n255\n",
        b"P5\n2 2\n255\n1 2 3 4\n",                   # binary magic: rejected
        b"P2#x\n2 2\n255\n1 2 3 4\n",                # magic runs to the space
        b"P2\n2 2\n255\n1 2 3\n",                    # short data
        b"P2\n2 2\n255\n1 2 x 4\n",                  # malformed value
        b"P2\nx 2\n255\n1 2 3 4\n",                  # malformed size
        b"",
    ]


def _mat2gray_cases():
    rng = np.random.default_rng(41)
    sino = (rng.standard_normal((45, 30)) * 40 + 10).astype(np.float32)
    pos = rng.random((19, 23)).astype(np.float32) * 3.5
    nan = pos.copy()
    nan[3, 4] = np.nan
    neg = -pos
    return [sino, pos, nan, neg, np.zeros((4, 3), np.float32),
            np.array([[1e-30, 2e-30], [3e-30, 0.0]], np.float32)]


def main_io():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    out = {}
    for i, ((r, c, seed), (orow, ocol)) in enumerate(RESIZE_CASES):
        img = _resize_input(r, c, seed)
        out[f"resize{i}_in"] = img
        out[f"resize{i}_out"] = O.ref_resize(img, orow, ocol)
    for i, text in enumerate(_pgm_cases()):
        out[f"pgm{i}_in"] = np.frombuffer(text, np.uint8)
        res = O.ref_netpbm(text)
        if "error" in res:
            out[f"pgm{i}_error"] = np.frombuffer(res["error"].encode(), np.uint8)
            continue
        for c in range(len(res["pixels"])):
            out[f"pgm{i}_c{c}_pixels"] = res["pixels"][c]
            out[f"pgm{i}_c{c}_gray"] = res["gray"][c]
            out[f"pgm{i}_c{c}_written"] = np.frombuffer(res["pgm"][c], np.uint8)
    for i, m in enumerate(_mat2gray_cases()):
        gray, text = O.ref_mat2gray(m)
        out[f"m2g{i}_in"] = np.asfortranarray(m)
        out[f"m2g{i}_out"] = gray
        out[f"m2g{i}_written"] = np.frombuffer(text, np.uint8)
    np.savez_compressed(os.path.join(HERE, "image_io.npz"), **out)
    print("image_io", len(out), "arrays")


if __name__ == "__main__":
    if sys.argv[1:] == ["io"]:
        main_io()
    else:
        main()
