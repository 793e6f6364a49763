"""The .cdb reader of tests/golden/make_golden.py and the BENCH fixtures it
wrote: re-reading the reference's test inputs gives the committed arrays
(skipped where the reference checkout is absent), and the fixtures are
well-formed models (every fixed DoF and CE term on a node of an element)."""
import os

import numpy as np
import pytest

import make_golden as mgd

GOLDEN = os.path.dirname(mgd.__file__)
from oracle.oracle import REF_TEST  # noqa: E402


@pytest.mark.skipif(not os.path.isdir(REF_TEST), reason="reference tests not present")
def test_damper_fixture_matches_a_fresh_read():
    md = mgd.read_cdb(f"{REF_TEST}/3d_damper/model.cdb")
    g = np.load(os.path.join(GOLDEN, "damper_3d.npz"))
    conn = np.array([c for c, t in zip(md["cells"], md["type"]) if t == 1], dtype=np.uint32)
    assert np.array_equal(conn, g["conn"]) and np.array_equal(md["xyz"], g["xyz"])
    assert len(md["mpcs"]) == g["mpc_b"].size == 497
    assert np.array_equal(np.array(md["comps"]["TOP_SIDE"]), g["top_side"])


@pytest.mark.skipif(not os.path.isdir(REF_TEST), reason="reference tests not present")
def test_a2000_fixture_matches_a_fresh_read():
    md = mgd.read_cdb(f"{REF_TEST}/a2000_damper/a2000.cdb")
    g = np.load(os.path.join(GOLDEN, "a2000_plane41.npz"))
    conn = np.array([c for c, t in zip(md["cells"], md["type"]) if t == 1], dtype=np.uint32)
    assert np.array_equal(conn, g["conn"]) and np.array_equal(md["xyz"], g["xyz"])
    assert np.array_equal(np.array([f[2] for f in md["fixes"]]), g["fix_value"])


@pytest.mark.parametrize("name", ["damper_3d", "a2000_plane41"])
def test_bench_fixtures_are_well_formed(name):
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    n_nodes = g["xyz"].shape[0]
    used = np.zeros(n_nodes + 1, bool)
    used[g["conn"].ravel()] = True
    assert g["conn"].min() >= 1 and g["conn"].max() <= n_nodes
    assert used[g["fix_node"]].all()
    if "mpc_node" in g.files:
        assert used[g["mpc_node"]].all()
        assert g["mpc_ptr"][-1] == g["mpc_node"].size
    assert g["ref_curve"].size == 21
