"""The drop-in simpleML compiles against the reference's own headers and the
reference's treeator.cpp relinks with it unchanged (CPU only; needs the
reference sources, so it is skipped where they are absent)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
from oracle import refpath

REFSRC = refpath.REF_SRC
EXAMPLES = refpath.REF_EXAMPLES


@pytest.mark.skipif(not os.path.isdir(REFSRC), reason="reference sources absent")
def test_treeator_relinks_against_dropin(tmp_path):
    out = tmp_path / "build"
    res = subprocess.run(["make", "-s", "-j8", "-C", os.path.join(ROOT, "phylommand_gb300", "dropin"),
                          f"REFSRC={REFSRC}", f"OUT={out}"], capture_output=True, text=True)
    assert res.returncode == 0, res.stdout + res.stderr
    exe = out / "treeator_gpu"
    assert exe.exists()
    # the relinked CLI runs and reaches the engine (without a GPU the engine
    # reports that and the drop-in returns 0.0, as the reference does on error)
    run = subprocess.run([str(exe), "-f", os.path.join(EXAMPLES, "alignment_file.fst"), "-t",
                          os.path.join(EXAMPLES, "tree_file.tree"), "-l", "-m", "0,0,0,0,0,0", "-P", "1.0",
                          "-F", ".25,.25,.25,.25", "-N"], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0
    assert "Log likelihood=" in run.stdout
