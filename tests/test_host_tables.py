"""Host-side bookkeeping of the product (no GPU): orbit order, channel kets,
cross-coupled kets, arena layout and the 6j table, against the reference's own
tables (golden fixtures) and the Python restatement."""
import numpy as np
import pytest

import imsrg_gb300 as ig
from helpers import load_golden
from modelspace_ref import RefModelSpace, read_ref_tables


@pytest.mark.parametrize("emax", [2, 3])
def test_tables_match_reference_dump(emax, tmp_path):
    g = load_golden(emax)
    p = tmp_path / "tables.txt"
    p.write_text(str(g["tables"]))
    t = read_ref_tables(str(p))
    ms = ig.ModelSpace(emax, "O16", "O16")
    assert [o[:4] for o in ms.orbits] == [o[:4] for o in t["orbits"]]
    assert [o[4] for o in ms.orbits] == [o[4] for o in t["orbits"]]
    for c in range(ms.nch):
        J, par, Tz, kets, cls = t["channels"][c]
        assert (ms.channels[c]["J"], ms.channels[c]["parity"], ms.channels[c]["Tz"]) == (J, par, Tz)
        assert ms.channels[c]["kets"] == kets
        cc = ms.cc_channel(c)
        assert cc["kets"] == t["cc_channels"][c][3]


@pytest.mark.parametrize("emax", [4, 6, 10])
def test_tables_match_restatement(emax):
    ms = ig.ModelSpace(emax, "O16", "O16")
    r = RefModelSpace(emax)
    assert ms.arena_size == r.arena_size
    for c in range(ms.nch):
        assert ms.channels[c]["kets"] == r.channels[c][3]
        assert ms.channels[c]["offset"] == r.off2[c]


def test_channel_sizes_emax10():
    ms = ig.ModelSpace(10, "O16", "O16")
    dims = [c["nkets"] for c in ms.channels]
    assert max(dims) == 1341
    assert max(ms.cc_channel(c)["nkets"] for c in range(ms.nch)) == 1386
    assert ms.norb == 132


def test_explicit_orbit_list_equals_reference_space():
    r = RefModelSpace(3)
    ms = ig.ModelSpace(3, orbits=(r.n, r.l, r.j2, r.tz2, r.occ))
    ms2 = ig.ModelSpace(3, "O16", "O16")
    assert ms.channels == ms2.channels


def test_bad_orbits_rejected():
    with pytest.raises(ig.IMSRGError):
        ig.ModelSpace(2, orbits=([0], [0], [2], [1], [1.0]))  # even j2


def test_parse_reference():
    assert ig.parse_reference("O16") == (16, 8)
    assert ig.parse_reference("Ca48") == (48, 20)
    assert ig.parse_reference("He4") == (4, 2)
