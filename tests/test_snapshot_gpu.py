"""Checkpoint/resume through binary snapshots, and the device-side initial field."""
import numpy as np
import pytest

from cns_nospec_gb300 import initdata as I

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [0, 1])
def test_resume_from_snapshot_is_bitwise(gpu, cns, tmp_path, prec):
    n = (20, 16, 24)
    dx = I.box_dx(n)
    U0 = I.initial_state(n, perturb=1e-3, seed=12)
    a = cns.Box(n, dx, I.CFL, I.ETA, I.ALAM, precision=prec)
    a.upload(U0)
    a.advance(8)
    ref = a.download()
    b = cns.Box(n, dx, I.CFL, I.ETA, I.ALAM, precision=prec)
    b.upload(U0)
    b.advance(3)
    b.save(tmp_path / "snap.bin")
    b.close()
    c = cns.Box(n, dx, I.CFL, I.ETA, I.ALAM, precision=prec)
    c.load(tmp_path / "snap.bin")
    assert c.last_dt()[1] == 3
    c.advance(5)
    assert np.array_equal(c.download(), ref)
    assert c.last_dt()[1] == 8


def test_snapshot_rejects_other_boxes(gpu, cns, tmp_path):
    n = 16
    a = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    a.init_field()
    a.save(tmp_path / "s.bin")
    b = cns.Box(n, I.box_dx(n), I.CFL, I.ETA * 2, I.ALAM)
    with pytest.raises(cns.CnsError):
        b.load(tmp_path / "s.bin")
    c = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM, precision=1)
    with pytest.raises(cns.CnsError):
        c.load(tmp_path / "s.bin")
    (tmp_path / "t.bin").write_bytes(b"garbage")
    with pytest.raises(cns.CnsError):
        a.load(tmp_path / "t.bin")


def test_device_initial_field_matches_host_generator(gpu, cns):
    n = (24, 20, 28)
    amp = (0.9, 1.1, 1.2)
    box = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM)
    box.init_field(amp=amp, perturb=1e-3, seed=77)
    D = box.download()
    H = I.initial_state(n, amp=amp, perturb=1e-3, seed=77)
    rel = np.abs(D - H) / np.abs(H).reshape(-1, 5).max(axis=0)
    assert rel.max() < 1e-14
