"""Host-side spectrum input (no GPU): the reference's cumulative half-keV
tables (monte_cu/CBCT_real325.cu:349-389, sampled at :479-486) into line
weights, and the text parser of those tables."""
import numpy as np

from monte_gb300 import lib


def _brute_force(cum, bin_kev, fallback, n=200_001):
    """The reference's loop on a fine grid of u in (0, 1]."""
    u = (np.arange(n) + 1.0) / n
    out = np.full(n, fallback)
    done = np.zeros(n, bool)
    for d in range(len(cum) - 1):
        hit = (~done) & (cum[d] <= u) & (u <= cum[d + 1])
        out[hit] = (d + 1) * bin_kev
        done |= hit
    return out


def test_cumulative_table_weights_match_the_reference_loop():
    rng = np.random.default_rng(5)
    tables = [
        np.concatenate([[0.0], np.cumsum(rng.random(20))]) / 20.0,   # monotone, ends < 1
        np.concatenate([[0.1], np.sort(rng.random(20))]),            # starts above 0
        rng.random(21),                                              # not monotone
        np.zeros(21),                                                # the reference's own state
    ]
    for cum in tables:
        cum = cum.astype(np.float32)
        E, W = lib.spectrum_from_cumulative(cum, 0.5, 140.0)
        assert len(E) == 21 and abs(W.sum() - 1.0) < 1e-12
        got = _brute_force(cum.astype(np.float64), 0.5, 140.0)
        for e, w in zip(E, W):
            frac = float(np.mean(got == e))
            assert abs(frac - w) < 2e-5, (e, frac, w)


def test_parse_numbers_reads_whitespace_tables():
    vals = lib.parse_numbers(b"0\n0.25\t0.5\r\n  1e-0 \n")
    assert np.array_equal(vals, np.array([0.0, 0.25, 0.5, 1.0], np.float32))
    assert lib.parse_numbers(b"").size == 0
