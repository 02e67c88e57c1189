"""The C ABI from a plain C program: phylommand_gb300/lib/plk_replay (built
by the package build from phylommand_gb300/capi/plk_replay.c, linked against
include/plk.h and libplk.so only) replays a golden fixture made by the
reference's own simpleML -- the set-up, lnL and node-state calls treeator
makes (src/treeator.cpp:715-724, :916, :973) -- and its results are held to
the reference's values."""
import os
import struct
import subprocess

import numpy as np
import pytest

from phylommand_gb300 import build, plk
import helpers as H


def _write_input(path, fx):
    masks = np.ascontiguousarray(fx["masks"], dtype=np.uint32)
    n_tips, n_sites = masks.shape
    S = int(fx["n_states"])
    C = len(fx["cat_rates"])
    with open(path, "wb") as f:
        f.write(struct.pack("<8i", n_tips, n_sites, S, len(fx["left"]), C, int(fx["root_quirk"]), int(fx["tr"]),
                            plk.PLK_P_TAYLOR20))
        f.write(masks.tobytes())
        f.write(np.ascontiguousarray(fx["left"], dtype="<i4").tobytes())
        f.write(np.ascontiguousarray(fx["right"], dtype="<i4").tobytes())
        for k in ("bl", "Q", "root_w", "cat_rates", "cat_weights"):
            f.write(np.ascontiguousarray(fx[k], dtype="<f8").tobytes())
    return n_sites, S


def test_replay_program_is_a_plain_c_caller():
    """Built, and linked against libplk only (no CUDA or Python library)."""
    assert os.path.exists(build.REPLAY)
    res = subprocess.run([build.REPLAY], capture_output=True, text=True)
    assert res.returncode == 2 and "usage" in res.stderr
    with open(build.REPLAY, "rb") as f:
        blob = f.read()
    assert b"libplk.so" in blob and b"libcudart" not in blob and b"libpython" not in blob


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["cfg1_jc16x1000", "quirk_b"])
def test_c_program_replays_reference_fixture(tmp_path, name):
    fx = H.load_fixture(name)
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    n_sites, S = _write_input(inp, fx)
    res = subprocess.run([build.REPLAY, str(inp), str(out)], capture_output=True, text=True)
    assert res.returncode == 0, res.stdout + res.stderr
    raw = out.read_bytes()
    lnl64, lnl32 = struct.unpack_from("<2d", raw, 0)
    (n_int,) = struct.unpack_from("<i", raw, 16)
    nodes = np.frombuffer(raw, dtype="<f8", count=n_int * n_sites * S, offset=20).reshape(n_int, n_sites, S)
    sites = np.frombuffer(raw, dtype="<f8", count=n_sites, offset=20 + 8 * n_int * n_sites * S)
    ref = float(fx["lnl"])
    assert abs(lnl64 - ref) <= 1e-12 * abs(ref)
    assert abs(lnl32 - ref) <= 1e-6 * abs(ref)
    np.testing.assert_allclose(sites, fx["site_lnl"], rtol=1e-12, atol=0)
    k = fx["node_cond"].shape[1]
    np.testing.assert_allclose(nodes[:, :k], H.normalise_cond(fx["node_cond"], fx["cat_weights"]), rtol=0, atol=1e-14)
