"""The reference's file formats (general_input, read_3D component files, print_4D dumps)
through the library's native readers/writers, checked against the reference's own I/O
functions where the reference tree is present (byte-identical dumps)."""
import os

import numpy as np
import pytest

from cns_nospec_gb300 import initdata as I


def _state(n=(5, 6, 7), seed=3):
    return I.initial_state(n, perturb=1e-3, seed=seed)


def test_print_4d_round_trip_is_exact(cns, tmp_path):
    from cns_nospec_gb300 import io
    U = _state()
    p = tmp_path / "output"
    io.print_4d(p, U, header=True)
    V = io.read_4d(p, U.shape[:3], 5, header=True)
    assert np.array_equal(U, V)
    with open(p) as f:
        assert f.readline().strip() == "5"
        assert f.readline().split() == [str(x) for x in U.shape[:3]]


def test_print_4d_is_byte_identical_to_reference(cns, oracle, tmp_path):
    if not oracle.have_ref():
        pytest.skip("reference tree not present")
    from cns_nospec_gb300 import io
    U = _state()
    ours, theirs = tmp_path / "a", tmp_path / "b"
    io.print_4d(ours, U, header=False)
    oracle.ref_print_4d(theirs, U)
    assert ours.read_bytes() == theirs.read_bytes()


def test_component_file_round_trip_and_reference_reader(cns, oracle, tmp_path):
    from cns_nospec_gb300 import io
    U = _state(seed=4)
    p = tmp_path / "multistep_input"
    io.write_3d(p, U)
    assert np.array_equal(io.read_3d(p, U.shape[:3], 5), U)
    if oracle.have_ref():
        assert np.array_equal(oracle.ref_read_3d(p, U.shape[:3], 5), U)


def test_general_input_matches_reference_reader(cns, oracle, tmp_path):
    from cns_nospec_gb300 import _lib as L
    from cns_nospec_gb300 import io
    h = cns.read_configurations((12, 10, 8), (0.1, 0.125, 0.0625), 0.5, 1.8e-4, 150.0, nsteps=7)
    h.dt = 3.25e-7
    os.makedirs(tmp_path / "testcases")
    os.makedirs(tmp_path / "run")
    io.write_general_input(tmp_path / "testcases" / "general_input", h)
    g = io.read_general_input(tmp_path / "testcases" / "general_input")
    for f, _ in L.GlobalConst._fields_:
        if f != "temp":
            a, b = getattr(h, f), getattr(g, f)
            assert (list(a) == list(b)) if hasattr(a, "__len__") else a == b, f
    if oracle.have_ref():
        r = L.GlobalConst()
        oracle.ref_read_configurations(tmp_path / "run", r)
        for f, _ in L.GlobalConst._fields_:
            if f != "temp":
                a, b = getattr(g, f), getattr(r, f)
                assert (list(a) == list(b)) if hasattr(a, "__len__") else a == b, f


def test_readers_reject_short_or_mismatched_files(cns, tmp_path):
    from cns_nospec_gb300 import io
    p = tmp_path / "bad"
    p.write_text("1 2 3\n")
    with pytest.raises(cns.CnsError):
        io.read_3d(p, (2, 2, 2), 1)
    with pytest.raises(cns.CnsError):
        io.read_general_input(p)
    U = _state()
    io.print_4d(p, U, header=True)
    with pytest.raises(cns.CnsError):
        io.read_4d(p, (5, 6, 8), 5, header=True)
    with pytest.raises(cns.CnsError):
        io.read_3d(tmp_path / "missing", (2, 2, 2), 1)
