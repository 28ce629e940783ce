"""The head of stdout0.out (elliptic::Print_Info: the run's parameters and
every box) written by Olliptic_gpu.x is the reference's, character for
character (tests/golden/banner, from its Olliptic.x).  It is written before
the device is touched, so no GPU is needed: the run is pointed at a device
that does not exist and stops after the banner."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "ollipticid_gb300", "_build", "Olliptic_gpu.x")
G = np.load(os.path.join(ROOT, "tests", "golden", "banner", "banners.npz"))
CASES = sorted({k.split("__")[0] for k in G.files})


@pytest.mark.parametrize("case", CASES)
def test_banner_is_the_references(case, tmp_path):
    from ollipticid_gb300 import build
    build.build()
    args = G[case + "__args"].item().decode()
    subprocess.run([CLI] + args.split() + ["-o", "Output", "-p1d", "no", "-pint", "no", "-gpu-device", "9999"],
                   cwd=str(tmp_path), capture_output=True, text=True, timeout=120)
    text = (tmp_path / "Output" / "stdout0.out").read_text()
    want = G[case + "__banner"].item().decode()
    assert text[:len(want)] == want
