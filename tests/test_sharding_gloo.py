"""Sharding of the transform over ranks (tracetransform_gb300/sharding.py):
the partitioning helpers, and one image's angles split over two gloo ranks on
the CPU.  The per-rank work is the oracle here (the engine needs a GPU), so
the test checks what sharding adds -- ranges, gather order, the z-score on
rank 0 -- by comparing the two-rank result with the oracle's own unsharded
transform, which it must equal bit for bit (every sinogram column and circus
entry depends on its own angle only)."""
import json
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

from tracetransform_gb300 import sharding

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_angle_ranges_cover_in_order():
    for n, w in [(360, 1), (360, 2), (360, 7), (5, 8), (0, 3), (720, 8)]:
        rs = sharding.angle_ranges(n, w)
        assert len(rs) == w and rs[0][0] == 0 and rs[-1][1] == n
        assert all(a[1] == b[0] for a, b in zip(rs, rs[1:]))
        sizes = [hi - lo for lo, hi in rs]
        assert max(sizes) - min(sizes) <= 1 and sum(sizes) == n
    with pytest.raises(ValueError):
        sharding.angle_ranges(10, 0)


def test_assign_images_greedy_by_cost():
    costs = [sharding.image_cost(r, c, a) for r, c, a in
             [(512, 512, 360), (64, 64, 180), (300, 200, 360), (512, 400, 360), (100, 100, 360)]]
    ranks = sharding.assign_images(costs, 2)
    assert sorted(i for r in ranks for i in r) == list(range(5))
    load = [sum(costs[i] for i in r) for r in ranks]
    # largest first: 0 -> rank 0, 3 -> rank 1, then the rest onto the lighter
    assert 0 in ranks[0] and 3 in ranks[1]
    assert max(load) <= sum(costs) / 2 + max(costs)
    assert sharding.assign_images([], 3) == [[], [], []]


_RANK_SCRIPT = r"""
import json, os, sys
sys.path.insert(0, os.environ["TT_ROOT"])
import numpy as np
import torch.distributed as dist
from oracle import oracle as O
from tracetransform_gb300 import sharding
from tracetransform_gb300.synthetic import blob_image


class OracleCompute:
    def sinograms(self, image, angles, tfs):
        return O.sinograms(O.pad(image), angles, list(tfs))
    def circus(self, sino, pfs):
        return np.stack([O.circus(s, [tuple(p) for p in pfs]) for s in sino])
    def zscore(self, v):
        return np.stack([O.zscore(x) for x in v])
    def orthonormal(self, sino, orders):
        out = []
        for s in sino:
            nos, c = O.nos(s)
            out.append(O.circus(nos, [(0, o, c) for o in orders]))
        return np.stack(out)


    def transform_images(self, images, steps, tfs, pfs):
        out = []
        for im, st in zip(images, steps):
            r = O.transform(im, int(st), list(tfs), [(k, o) for k, o, _ in pfs])
            out.append((r["circus"], np.ascontiguousarray(r["sig"])))
        return out


rank, world = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
dist.init_process_group("gloo")
O.build()
img = blob_image(40, 32, 5, (3, 10), (40, 200), 7)
res = {}
for name, step, tfs, pfs in [("regular", 4, [0, 1, 5, 6, 7], [(1, 0, -1), (2, 0, -1), (3, 0, -1)]),
                             ("hermite", 6, [0, 2], [(0, 1, -1), (0, 3, -1)])]:
    r = sharding.transform_angle_sharded(img, step, tfs, pfs, rank, world,
                                         compute=OracleCompute())
    if rank == 0:
        np.save(os.path.join(os.environ["TT_OUT"], name + "_circus.npy"), r[0])
        np.save(os.path.join(os.environ["TT_OUT"], name + "_sig.npy"), r[1])
    else:
        assert r is None
imgs = [blob_image(r, c, 3, (2, 6), (40, 200), 50 + i)
        for i, (r, c) in enumerate([(20, 14), (33, 30), (12, 25), (28, 28), (16, 16)])]
steps = [6, 4, 8, 6, 5]
res = sharding.transform_images_sharded(imgs, steps, [0, 2, 7], [(1, 0, -1), (3, 0, -1)],
                                        rank, world, compute=OracleCompute())
if rank == 0:
    for i, (c, z) in enumerate(res):
        np.save(os.path.join(os.environ["TT_OUT"], "batch%d_circus.npy" % i), c)
        np.save(os.path.join(os.environ["TT_OUT"], "batch%d_sig.npy" % i), z)
else:
    assert res is None
dist.destroy_process_group()
print(json.dumps({"rank": rank, "ok": True}))
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_angle_sharded_transform_two_gloo_ranks(oracle_lib, tmp_path):
    O = oracle_lib
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2",
                   RANK=str(rank), LOCAL_RANK=str(rank), TT_ROOT=ROOT, TT_OUT=str(tmp_path))
        procs.append(subprocess.Popen([sys.executable, "-c", _RANK_SCRIPT], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    try:
        for p in procs:
            out, err = p.communicate(timeout=300)
            assert p.returncode == 0, err
            assert json.loads(out.strip().splitlines()[-1])["ok"]
    finally:
        for p in procs:  # a rank that failed or hung must not outlive the test
            if p.poll() is None:
                p.kill()
                p.wait()
    from tracetransform_gb300.synthetic import blob_image
    img = blob_image(40, 32, 5, (3, 10), (40, 200), 7)
    # regular mode: the oracle's unsharded Transformer
    want = O.transform(img, 4, [0, 1, 5, 6, 7], [(O.P1, 0), (O.P2, 0), (O.P3, 0)])
    got_c = np.load(tmp_path / "regular_circus.npy")
    got_s = np.load(tmp_path / "regular_sig.npy")
    assert np.array_equal(got_c.view(np.uint32), want["circus"].view(np.uint32))
    assert np.array_equal(got_s.view(np.uint32), np.asarray(want["sig"]).view(np.uint32))
    # orthonormal mode on the unstretched image: every sinogram gathered on
    # rank 0, nearest orthonormal sinogram and Hermite there
    sino = O.sinograms(O.pad(img), O.angles_for_step(6), [0, 2])
    herm = []
    for s in sino:
        nos, c = O.nos(s)
        herm.append(O.circus(nos, [(0, 1, c), (0, 3, c)]))
    herm = np.stack(herm)
    got_h = np.load(tmp_path / "hermite_circus.npy")
    assert np.array_equal(got_h.view(np.uint32), herm.view(np.uint32))
    z = np.stack([O.zscore(v) for v in herm.reshape(-1, herm.shape[2])])
    assert np.array_equal(np.load(tmp_path / "hermite_sig.npy").view(np.uint32),
                          np.ascontiguousarray(z.T).view(np.uint32))
    # a batch over the two ranks: every image's result back on rank 0, in order
    for i, ((r, c), st) in enumerate(zip([(20, 14), (33, 30), (12, 25), (28, 28), (16, 16)],
                                         [6, 4, 8, 6, 5])):
        im = blob_image(r, c, 3, (2, 6), (40, 200), 50 + i)
        w = O.transform(im, st, [0, 2, 7], [(O.P1, 0), (O.P3, 0)])
        assert np.array_equal(np.load(tmp_path / ("batch%d_circus.npy" % i)), w["circus"])
        assert np.array_equal(np.load(tmp_path / ("batch%d_sig.npy" % i)), np.asarray(w["sig"]))

