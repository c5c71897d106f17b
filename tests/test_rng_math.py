"""Random streams and elementary functions shared by the kernels and the
CPU replay harness (monte_gb300/csrc/monte_rng.h)."""
import numpy as np

import oracle


def test_philox_known_answers():
    # Random123 known-answer vectors for philox4x32-10
    cases = [
        ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
        ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF), (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
        ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
         (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
    ]
    for ctr, key, want in cases:
        assert tuple(int(v) for v in oracle.philox(ctr, key)) == want


def test_uniform_range_and_moments():
    u = oracle.stream(1234, 99, 0, 1 << 20)
    assert u.min() > 0.0 and u.max() <= 1.0
    assert abs(u.mean() - 0.5) < 2e-3
    assert abs(u.var() - 1.0 / 12) < 1e-3
    # distinct histories and jobs give distinct streams
    assert not np.array_equal(oracle.stream(1234, 100, 0, 64), oracle.stream(1234, 99, 0, 64))
    assert not np.array_equal(oracle.stream(1234, 99, 1, 64), oracle.stream(1234, 99, 0, 64))


def test_logf_accuracy():
    k = np.arange(1, 1 << 24, 97, dtype=np.float64)
    x = (k * 2.0 ** -24).astype(np.float32)
    y = oracle.logf(x).astype(np.float64)
    ref = np.log(x.astype(np.float64))
    ulp = np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
    err = np.abs(y - ref) / np.maximum(ulp, 1e-45)
    assert err.max() < 2.0, err.max()


def test_sincos_accuracy():
    u = (np.arange(0, 1 << 24, 13, dtype=np.float64) * 2.0 ** -24).astype(np.float32)
    s, c = oracle.sincos_2pi(u)
    a = 2 * np.pi * u.astype(np.float64)
    assert np.abs(s - np.sin(a)).max() < 1.5e-7
    assert np.abs(c - np.cos(a)).max() < 1.5e-7
