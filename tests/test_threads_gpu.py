"""Calls from several host threads at once: each thread's host-array advances (its own cached
box and stream) and its own device-resident boxes give the same bits as the same calls made
one after another.  ctypes releases the GIL around each foreign call, so the calls overlap."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _work(cns, I, n, precision, seed, out, key):
    U = I.initial_state(n, perturb=1e-3, seed=seed)
    dts = cns.advance_host(U, 3, I.box_dx(n), I.CFL, I.ETA, I.ALAM, precision)
    box = cns.Box(n, I.box_dx(n), I.CFL, I.ETA, I.ALAM, precision=precision)
    try:
        box.upload(I.initial_state(n, perturb=1e-3, seed=seed + 1))
        box.advance(4)
        V = box.download()
        box.sync()
    finally:
        box.close()
    out[key] = (U, dts, V)


CASES = [((24, 20, 28), 0, 3), ((20, 24, 16), 1, 5), ((16, 16, 40), 0, 7), ((28, 12, 20), 1, 9)]


def test_concurrent_threads_equal_sequential(gpu, cns):
    from cns_nospec_gb300 import initdata as I
    seq = {}
    for q, (n, prec, seed) in enumerate(CASES):
        _work(cns, I, n, prec, seed, seq, q)
    par, errors = {}, []

    def run(q, n, prec, seed):
        try:
            for _ in range(3):  # several rounds, so that the threads' calls interleave
                _work(cns, I, n, prec, seed, par, q)
        except Exception as e:  # reported below; a thread's exception is not raised by join
            errors.append(repr(e))

    threads = [threading.Thread(target=run, args=(q,) + c) for q, c in enumerate(CASES)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not any(t.is_alive() for t in threads)
    assert not errors, errors
    for q in range(len(CASES)):
        for a, b in zip(seq[q], par[q]):
            assert np.array_equal(np.asarray(a).view(np.uint64), np.asarray(b).view(np.uint64)), CASES[q]
