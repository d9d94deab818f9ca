"""Receiver response functions and active source-receiver masks, applied to
sampled wavefields as recsub.f and makeuh.f do.

recsub.f builds one complex response per receiver and frequency:

  recin = 1  DFT of a time trace: r(f) = (1/nsam) sum_j trace_j exp(+i w t_j),
             with t_j = (j - 1) dt, dt in ms, and the start time forced to 0
             (recsub.f:95-102, 105-118).  The shipped reference returns an
             error before it reaches this branch (recsub.f:58-61); the
             definition is the one written there.
  recin = 3  unit response, a delta function (recsub.f:154-162).

makeuh.f multiplies the three geophone components by the response when
recin != 0 (makeuh.f:92-98) and zeroes the pairs that are not active
(sg = 0, makeuh.f:99-103).  Hydrophone pressures carry no response and are
zeroed for inactive pairs (sr = 0, makeuh.f:126, 165-166).

The arithmetic is a few multiplies per receiver, so it runs on the host after
wt3d_sample_receivers / wt3d_sample_pressure.
"""
import numpy as np


def response_from_traces(traces, dt_ms, freqs):
    """recin = 1: responses (nrec, nfreq) from time traces (nsam, nrec)
    sampled every dt_ms milliseconds from t = 0."""
    tr = np.asarray(traces, np.float64)
    if tr.ndim == 1:
        tr = tr[:, None]
    nsam = tr.shape[0]
    if nsam < 1:
        raise ValueError("response_from_traces: empty traces")
    t = np.arange(nsam) * (float(dt_ms) / 1000.0)
    w = 2.0 * np.pi * np.asarray(freqs, np.float64).reshape(-1)
    kernel = np.exp(1j * np.outer(t, w)) / nsam          # (nsam, nfreq)
    return tr.T @ kernel                                 # (nrec, nfreq)


def delta_response(nrec, nfreq):
    """recin = 3: unit responses (nrec, nfreq)."""
    return np.ones((int(nrec), int(nfreq)), np.complex128)


def apply_geophone_response(samples, response=None, active=None):
    """Geophone samples (nsrc, nrec, 3) at one frequency: times response[nrec]
    (None: recin = 0, unchanged) and zero where active[nsrc, nrec] is 0
    (None: every pair active)."""
    out = np.array(samples, np.complex128, copy=True)
    if out.ndim != 3 or out.shape[2] != 3:
        raise ValueError("apply_geophone_response: samples must be (nsrc, nrec, 3)")
    if response is not None:
        r = np.asarray(response, np.complex128).reshape(-1)
        if r.size != out.shape[1]:
            raise ValueError("apply_geophone_response: one response per receiver")
        out *= r[None, :, None]
    if active is not None:
        a = np.asarray(active).reshape(out.shape[0], out.shape[1])
        out[a == 0] = 0
    return out


def apply_hydrophone_mask(pressure, active=None):
    """Hydrophone pressures (nsrc, nrec): zero where active[nsrc, nrec] is 0."""
    out = np.array(pressure, np.complex128, copy=True)
    if active is not None:
        a = np.asarray(active).reshape(out.shape)
        out[a == 0] = 0
    return out
