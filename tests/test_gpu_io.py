"""Operator files (imsrg_op_write_binary / imsrg_op_read_binary, the
reference's Operator::WriteBinary / ReadBinary layout) and the solver's
scratch-file Omegas, on the GPU.  The files must interchange with the
reference: the reference's own files (golden fixtures) are read exactly, and
the files written here equal the reference's byte for byte apart from the
E2max field, which the reference writes from an uninitialised member."""
import os

import numpy as np
import pytest

import imsrg_gb300 as ig
from helpers import load_flow_golden, load_golden, rel_errors, ref_space

pytestmark = pytest.mark.gpu

E2MAX = slice(20, 24)  # bytes of the E2max field


@pytest.mark.parametrize("emax", [2, 3])
@pytest.mark.parametrize("name,herm", [("X", 1), ("Y", -1)])
def test_reads_reference_files(tmp_path, emax, name, herm):
    g = load_golden(emax)
    ms = ig.ModelSpace(emax, "O16", "O16")
    f = tmp_path / "op.bin"
    g[name + "_binary"].tofile(f)
    with ig.DeviceOperator(ms, 1) as d:
        d.upload(np.full(ms.arena_size, 7.0))  # padding must come back zero
        d.read_binary(str(f))
        assert d.hermiticity == herm
        assert np.array_equal(d.download(), g[name])


@pytest.mark.parametrize("emax", [2, 3])
@pytest.mark.parametrize("name,herm", [("X", True), ("Y", False)])
def test_writes_reference_layout(tmp_path, emax, name, herm):
    g = load_golden(emax)
    ms = ig.ModelSpace(emax, "O16", "O16")
    f = tmp_path / "op.bin"
    ig.Operator(ms, arena=g[name], hermitian=herm).WriteBinary(str(f))
    mine = np.fromfile(f, dtype=np.uint8)
    ref = g[name + "_binary"]
    assert mine.size == ref.size
    keep = np.ones(ref.size, bool)
    keep[E2MAX] = False
    assert np.array_equal(mine[keep], ref[keep])
    assert int.from_bytes(bytes(mine[E2MAX]), "little") == 2 * emax


def test_round_trip_many_chunks(tmp_path):
    # emax=10: 280 MiB, streamed through the staging buffers in several chunks
    ms = ig.ModelSpace(10, "O16", "O16")
    f = str(tmp_path / "big.bin")
    with ig.DeviceOperator(ms, -1) as a, ig.DeviceOperator(ms, 1) as b:
        a.fill_random(12345)
        a.write_binary(f)
        assert os.path.getsize(f) > 8 * 4 * (1 << 20)
        b.read_binary(f)
        assert b.hermiticity == -1
        assert np.array_equal(a.download(), b.download())


def test_rejects_mismatched_files(tmp_path):
    g = load_golden(2)
    f = tmp_path / "x.bin"
    g["X_binary"].tofile(f)
    ms3 = ig.ModelSpace(3, "O16", "O16")
    with ig.DeviceOperator(ms3, 1) as d:
        with pytest.raises(ig.IMSRGError):
            d.read_binary(str(f))
    ms2 = ig.ModelSpace(2, "O16", "O16")
    g["X_binary"][:-8].tofile(f)
    with ig.DeviceOperator(ms2, 1) as d:
        with pytest.raises(ig.IMSRGError):
            d.read_binary(str(f))
        with pytest.raises(ig.IMSRGError):
            d.read_binary(str(tmp_path / "missing.bin"))


def test_solver_scratch_omegas(tmp_path):
    # Omega splits written to scratch files give the same flow as Omegas kept
    # in device memory; Transform reads the files back
    g = load_flow_golden(3)
    ms = ig.ModelSpace(3, "O16", "O16")
    r = ref_space(3)
    H = ig.Operator(ms, arena=g["H"])

    def flow(scratch):
        sv = ig.IMSRGSolver(H, precision="fp64")
        if scratch:
            sv.SetScratchDir(scratch)
        sv.SetOmegaNormMax(0.3)
        sv.SetSmax(2.0)
        sv.Solve()
        return sv

    mem = flow(None)
    disk = flow(str(tmp_path))
    n_split = mem.GetOmegaSize() - 1
    assert n_split > 0
    assert disk.GetOmegaSize() == 1 and disk.GetNOmegaWritten() == n_split
    files = sorted(os.listdir(tmp_path))
    assert len(files) == n_split and all(x.startswith("OMEGA_") for x in files)
    Hm, Hd = mem.GetH_s(), disk.GetH_s()
    assert max(rel_errors(r, Hd.arena, Hm.arena)) < 1e-13
    T = disk.Transform(H)
    assert max(rel_errors(r, T.arena, Hd.arena)) < 1e-12
    disk.close()
    assert os.listdir(tmp_path) == []


# Tensor operators: the reference's Operator::WriteBinary of T (golden_tensor_*)
@pytest.mark.parametrize("emax,case", [(2, "e2"), (2, "e1"), (2, "gt"), (3, "e2")])
def test_tensor_files_interchange(tmp_path, emax, case):
    from helpers import load_tensor_golden
    g = load_tensor_golden(emax)
    lam, trank, par, herm = (int(x) for x in g[case + "_rank"])
    ms = ig.ModelSpace(emax, "O16", "O16")
    ref = g[case + "_binary"]
    f = tmp_path / "t.bin"
    ref.tofile(f)
    with ig.DeviceOperator(ms, 1, (lam, trank, par)) as d:
        d.upload(np.full(d.size, 7.0))  # padding must come back zero
        d.read_binary(str(f))
        assert d.hermiticity == herm
        assert np.array_equal(d.download(), g[case + "_T"])
        out = tmp_path / "mine.bin"
        d.write_binary(str(out))
    mine = np.fromfile(out, dtype=np.uint8)
    assert mine.size == ref.size
    keep = np.ones(ref.size, bool)
    keep[E2MAX] = False
    assert np.array_equal(mine[keep], ref[keep])
    # a file of another rank is refused
    with ig.DeviceOperator(ms, 1, (lam + 1, trank, par)) as d2:
        with pytest.raises(ig.IMSRGError):
            d2.read_binary(str(f))
