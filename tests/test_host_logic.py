"""Host-side logic of the drop-in: CFL/frame clock, reinit schedule, seeding and layouts (CPU)."""
import numpy as np
import pytest

import oracle as O
import pfm


def test_clock_matches_reference_rule():
    c = pfm.DtClock(CFL=0.5, dx=1 / 32, visualize_dt=0.1)
    dts = []
    for ms in (0.1, 0.1, 0.2, 5.0, 0.01):
        dt, out = c.next(ms)
        dts.append((dt, out))
    # first: 0.5/32/0.1 = 0.15625 >= 0.1 -> clamped to the frame end
    assert dts[0] == (pytest.approx(0.1), True)
    assert dts[2][0] == pytest.approx(0.078125) and not dts[2][1]
    assert dts[3][0] == pytest.approx(0.5 / 32 / 5.0) and not dts[3][1]
    assert c.sub_t == pytest.approx(0.078125 + 0.5 / 32 / 5.0 + 0.0 if not dts[4][1] else 0.0) or dts[4][1]


def test_clock_same_as_oracle():
    a, b = pfm.DtClock(0.5, 1 / 64, 0.1), O.DtClock(0.5, 1 / 64, 0.1)
    rng = np.random.default_rng(0)
    for ms in rng.uniform(0.05, 3.0, 200):
        assert a.next(ms) == b.next(ms)


def test_lattice_is_the_reference_order():
    p = pfm.lattice3((4, 3, 2), 0.25)
    assert p.shape == (4 * 3 * 2 * 8, 3)
    # x fastest: consecutive particles step by dx/2 in x (init_conditions.py:246-252)
    assert np.allclose(p[1] - p[0], [0.125, 0, 0])
    assert np.allclose(p[8], [0.0625, 0.1875, 0.0625])
    assert np.array_equal(p, O.lattice3((4, 3, 2), 0.25))
    assert np.array_equal(pfm.lattice2((8, 4), 0.25, 4), O.lattice2((8, 4), 0.25, 4))


def test_jitter_is_seeded_stratified_and_line_grouped():
    a = pfm.jittered((4, 4, 4), 0.25, 8, seed=0)
    b = pfm.jittered((4, 4, 4), 0.25, 8, seed=0)
    c = pfm.jittered((4, 4, 4), 0.25, 8, seed=1)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    cells = np.floor(a / 0.25).astype(int)
    lin = (cells[:, 0] * 4 + cells[:, 1]) * 4 + cells[:, 2]
    # each line of 4 cells along z holds its 32 particles consecutively, 8 per cell
    assert np.array_equal(lin // 4, np.repeat(np.arange(16), 32))
    assert np.array_equal(np.bincount(lin, minlength=64), np.full(64, 8))
    sub = np.floor(a / 0.125).astype(int) % 2
    for cell in range(64):  # one per sub-cell
        assert len({tuple(s) for s in sub[lin == cell]}) == 8
    # 32 consecutive particles of a 16-cell group: 16 cells along z, one leading sub-cell
    g = pfm.jittered((2, 2, 32), 1 / 32, 8, seed=0)
    gc = np.floor(g / np.float32(1 / 32)).astype(int)
    gs = np.floor(g / np.float32(1 / 64)).astype(int) % 2
    for w in range(4):
        blk = slice(32 * w, 32 * w + 32)
        assert len({tuple(s) for s in gs[blk, :2]}) == 1 and len(set(gc[blk, 2])) == 16
    two = pfm.jittered((8, 8), 1 / 8, 4, seed=0)
    assert two.shape == (256, 2)
    with pytest.raises(ValueError):
        pfm.jittered((4, 4), 0.25, 3)


def test_soa_round_trip():
    rng = np.random.default_rng(0)
    a = rng.standard_normal((10, 3)).astype(np.float32)
    T = rng.standard_normal((10, 3, 3)).astype(np.float32)
    s = pfm.soa(a, "cpu")
    assert tuple(s.shape) == (3, 10) and np.array_equal(pfm.aos(s), a)
    t = pfm.soa_T(T, "cpu")
    assert tuple(t.shape) == (3, 3, 10) and np.array_equal(pfm.aos_T(t), T)
    # element (v, c, q) is T_v[c] of particle q
    assert t[1, 2, 7] == T[7, 1, 2]


def test_reinit_schedule_3d_vs_2d():
    """3D resets ik only when particles are reseeded (run_3D.py:751-755); 2D always (run_2D.py:811-819)."""
    def sched(n, every, gm, is3d, reseed=True):
        out, ik = [], 0
        for i in range(n):
            j = i % every
            if j == 0:
                if is3d:
                    if reseed or i == 0:
                        ik = i
                else:
                    ik = i
            out.append((j == 0, (i - ik) % gm == 0))
        return out
    s3 = sched(12, 5, 2, True, reseed=False)
    assert [k for _, k in s3] == [(i % 2 == 0) for i in range(12)]
    s2 = sched(12, 5, 2, False)
    assert s2[5] == (True, True) and s2[6] == (False, False) and s2[7] == (False, True)


def test_solve_option_warm_start_values():
    """Scene._opts maps the Python warm_start values to the C field (False/True -> 0/1, 2 and 3 as
    given) and rejects anything else on the host."""
    import pfm
    from pfm.core import Scene
    for v, want in ((False, 0), (True, 1), (0, 0), (1, 1), (2, 2), (3, 3), (None, 0)):
        assert Scene._opts(400, 1e-6, 2, 4, warm_start=v).warm_start == want, v
    for bad in (4, -1, "quad"):
        with pytest.raises(pfm.PfmError):
            Scene._opts(400, 1e-6, 2, 4, warm_start=bad)
