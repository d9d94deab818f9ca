"""Receiver responses and active-pair masks (recsub.f, makeuh.f) on the host."""
import numpy as np
import pytest

from wtomo3d_gb300 import receivers


def loop_response(traces, dt_ms, freqs):
    """recsub.f:105-118 written as its loops."""
    nsam, nrec = traces.shape
    out = np.zeros((nrec, len(freqs)), np.complex128)
    for i in range(nrec):
        for f, fr in enumerate(freqs):
            w = 2 * np.pi * fr
            for j in range(nsam):
                t = j * dt_ms / 1000.0
                out[i, f] += traces[j, i] * np.exp(1j * w * t) / nsam
    return out


def test_impulse_responses():
    nsam, dt = 64, 4.0
    freqs = [0.5, 1.0, 2.0, 7.5]
    tr = np.zeros((nsam, 2))
    tr[0, 0] = 1.0               # impulse at t = 0: flat 1/nsam
    tr[10, 1] = 1.0              # delayed impulse: phase exp(+i w t0)
    r = receivers.response_from_traces(tr, dt, freqs)
    np.testing.assert_allclose(r[0], np.full(len(freqs), 1.0 / nsam), atol=1e-15)
    t0 = 10 * dt / 1000.0
    np.testing.assert_allclose(r[1], np.exp(1j * 2 * np.pi * np.array(freqs) * t0) / nsam, rtol=1e-13)


def test_response_matches_loops_and_is_linear():
    rng = np.random.default_rng(4)
    tr = rng.standard_normal((50, 3))
    freqs = [0.3, 1.1, 2.0]
    r = receivers.response_from_traces(tr, 2.0, freqs)
    np.testing.assert_allclose(r, loop_response(tr, 2.0, freqs), rtol=1e-12, atol=1e-15)
    r2 = receivers.response_from_traces(2.0 * tr + 1.0, 2.0, freqs)
    r1 = receivers.response_from_traces(np.ones_like(tr), 2.0, freqs)
    np.testing.assert_allclose(r2, 2.0 * r + r1, rtol=1e-12, atol=1e-14)


def test_delta_response_and_masks():
    np.testing.assert_array_equal(receivers.delta_response(3, 2), np.ones((3, 2)))
    rng = np.random.default_rng(5)
    s = rng.standard_normal((2, 4, 3)) + 1j * rng.standard_normal((2, 4, 3))
    resp = np.array([1.0, 2j, -1.0, 0.5])
    act = np.array([[1, 1, 0, 1], [0, 1, 1, 1]])
    out = receivers.apply_geophone_response(s, resp, act)
    for i in range(2):
        for r in range(4):
            want = s[i, r] * resp[r] if act[i, r] else np.zeros(3)
            np.testing.assert_allclose(out[i, r], want, rtol=1e-15)
    # recin = 0: unchanged; all pairs active
    np.testing.assert_array_equal(receivers.apply_geophone_response(s), s)
    p = rng.standard_normal((2, 4)) + 0j
    pm = receivers.apply_hydrophone_mask(p, act)
    np.testing.assert_array_equal(pm, np.where(act != 0, p, 0))


def test_bad_shapes():
    with pytest.raises(ValueError):
        receivers.apply_geophone_response(np.zeros((2, 4)), None)
    with pytest.raises(ValueError):
        receivers.apply_geophone_response(np.zeros((2, 4, 3)), np.ones(3))
    with pytest.raises(ValueError):
        receivers.response_from_traces(np.zeros((0, 2)), 1.0, [1.0])
