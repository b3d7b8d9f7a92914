"""The drop-in link: IMSRG++ compiled from its own sources with
imsrg_gb300/shim/imsrg_gpu_shim.cc in place of Commutator::comm*ss,
CommutatorScalarScalar and BCH::Standard_BCH_Transform
(oracle/ref_build.mk, target shim; built by __graft_entry__.build() where the
reference sources exist, skipped elsewhere).

Without a GPU it checks what the link itself decides:
- through the shim, the GPU model space's channels and kets equal the
  reference ModelSpace's (the arena layout contract), emax 2 to 6;
- every replaced entry point, and the reference's own dispatchers above them
  (Commutator::Commutator, BCH::BCH_Transform), reach imsrg_gb300: with no GPU
  its calls fail with an "imsrg_gb300:" error, which the reference's own
  implementation would not raise."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "shim_harness")

pytestmark = pytest.mark.skipif(not os.path.exists(HARNESS), reason="the drop-in link is built only where the "
                                "reference sources exist")


@pytest.mark.parametrize("emax", [2, 4, 6])
def test_shim_layout_matches_reference_channels(emax):
    r = subprocess.run([HARNESS, "layout", str(emax)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "layout ok" in r.stdout


def test_reference_entry_points_dispatch_to_the_shim():
    import torch
    if torch.cuda.is_available():
        pytest.skip("with a GPU the calls succeed; this check reads the no-GPU failure")
    r = subprocess.run([HARNESS, "dispatch", "2"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = dict(ln.rsplit(" ", 1) for ln in r.stdout.splitlines() if ln.endswith((" imsrg_gb300", " reference")))
    names = ["comm110ss", "comm220ss", "comm111ss", "comm121ss", "comm122ss", "comm221ss", "comm222_pp_hhss",
             "comm222_pp_hh_221ss", "comm222_phss", "Commutator::Commutator", "BCH::BCH_Transform"]
    for n in names:
        assert lines.get(n) == "imsrg_gb300", (n, r.stdout)
