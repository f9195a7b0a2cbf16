"""The collision test's random streams (CPU, oracle).

Each step of a particle collides with probability P, independently of its
other steps. The test is drawn from Philox4x32-10 streams keyed by (particle
id, seed) in two parts (q = 1/256): the step is a candidate when its byte
(step & 15) of the block counted (step >> 4, draw 2) is zero; with P <= q it
collides iff a candidate and u_acc < 256 P (block (step, draw 3)), with P > q
iff a candidate or else u_f < (P - q) / (1 - q) (block (step, draw 4)).

Checked here: the oracle's decisions against a restatement of that rule on
the pinned Philox (tests/test_oracle_pins.py holds its known answers), the
collision rate against P on both sides of q (binomial, 5 sigma), the
independence of consecutive steps (the rate of colliding pairs against P^2),
and the kernels' sixteen-step candidate mask (philox.h candidate_mask, built
for the host) against the candidate bytes.
"""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]

import oracle as O

SEED = 0x1234_5678_9ABC_DEF0


def _u01(a, b):
    return (float(a >> 5) * 67108864.0 + float(b >> 6)) / 9007199254740992.0


def _block(count, draw, pid, seed):
    return O.philox([count & 0xFFFFFFFF, draw, count >> 32, seed >> 32], [pid, seed & 0xFFFFFFFF])


def _byte(step, pid, seed):
    b = _block(step >> 4, 2, pid, seed)
    k = step & 15
    return (int(b[k >> 2]) >> (8 * (k & 3))) & 0xFF


def _rule(step, pid, seed, P):
    """The decision rule written out on the oracle's Philox."""
    byte = _byte(step, pid, seed)
    q = 1.0 / 256.0
    if P <= q:
        if byte != 0:
            return False
        r = _block(step, 3, pid, seed)
        return _u01(int(r[0]), int(r[1])) < P * 256.0
    if byte == 0:
        return True
    r = _block(step, 4, pid, seed)
    return _u01(int(r[0]), int(r[1])) < (P - q) / (1.0 - q)


@pytest.mark.parametrize("P", [1e-4, 3.9e-3, 1.0 / 256.0, 0.02, 0.4])
def test_oracle_follows_the_rule(P):
    rng = np.random.default_rng(7)
    steps = rng.integers(0, 1 << 40, 3000, dtype=np.uint64)
    ids = rng.integers(0, 1 << 28, 3000, dtype=np.uint32)
    got = O.collides(steps, ids, SEED, P)
    want = np.array([_rule(int(s), int(i), SEED, P) for s, i in zip(steps, ids)])
    assert np.array_equal(got, want)
    # candidates are 1 step in 256: the candidates among 8,192 steps of one id
    # exercise the acceptance draw
    cs = np.array([s for s in range(8192) if _byte(s, 5, SEED) == 0], np.uint64)
    assert len(cs) > 10
    ci = np.full(len(cs), 5, np.uint32)
    got = O.collides(cs, ci, SEED, P)
    assert np.array_equal(got, np.array([_rule(int(s), 5, SEED, P) for s in cs]))
    if P < 1e-3:
        assert not got.all()
    if P > 1.0 / 256.0:
        assert got.all()


@pytest.mark.parametrize("P", [2e-4, 1e-3, 1.0 / 256.0, 0.01, 0.25])
def test_rate_and_independence(P):
    n_ids, n_steps = 200_000, 32
    ids = np.repeat(np.arange(n_ids, dtype=np.uint32), n_steps)
    steps = np.tile(np.arange(1000, 1000 + n_steps, dtype=np.uint64), n_ids)
    hit = O.collides(steps, ids, SEED, P).reshape(n_ids, n_steps)
    n = hit.size
    sd = np.sqrt(n * P * (1 - P))
    assert abs(hit.sum() - n * P) <= 5 * sd, (hit.sum(), n * P, sd)
    # every position in the sixteen-step block collides at the same rate
    per_pos = hit.reshape(n_ids, 2, 16).sum(axis=(0, 1))
    m = n_ids * 2
    assert np.all(np.abs(per_pos - m * P) <= 5 * np.sqrt(m * P * (1 - P)) + 2), per_pos
    # consecutive steps: P(both) = P^2
    pairs = (hit[:, :-1] & hit[:, 1:]).sum()
    npair = n_ids * (n_steps - 1)
    ep = npair * P * P
    assert abs(pairs - ep) <= 5 * np.sqrt(ep) + 3, (pairs, ep)


def test_candidate_mask_matches_candidate_bytes(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    exe = tmp_path / "candidate_mask_check"
    subprocess.run([gxx, "-O2", "-std=c++17", f"-I{ROOT / 'start_gb300' / 'csrc'}",
                    str(ROOT / "tests" / "native" / "candidate_mask_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), "1000000"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
    assert "mismatches 0" in out.stdout
