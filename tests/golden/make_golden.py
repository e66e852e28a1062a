"""Regenerate the golden fixtures in this folder from the reference itself.

Runs maleadt/tracetransform's own c++/ sources, compiled unmodified against
the stand-in headers in oracle/shim/ (``make -C oracle ref``; needs a checkout
of the reference, by default /root/reference), on seeded synthetic images and
stores inputs and outputs as compressed .npz files:

    python tests/golden/make_golden.py

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


if __name__ == "__main__":
    main()
