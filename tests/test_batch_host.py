"""Host-side logic of the batched quenches (no GPU): the seeded workload draw."""
import math

from dynamite_gb300.batch import MT19937_64, mixed_length_quenches


def test_mt19937_64_matches_the_standard():
    # [rand.predef]: the 10000th output of a default-constructed mt19937_64
    r = MT19937_64()
    for _ in range(9999):
        r()
    assert r() == 9981545732273789042


def test_mixed_length_workload():
    lengths, qs = mixed_length_quenches()
    assert lengths == [256, 512, 1024] and len(qs) == 64
    assert {q.lam for q in qs} == {0.3, 0.5, 0.7}
    assert qs[0].Gamma == 0.4 and abs(qs[-1].Gamma - 1.0) < 1e-15
    assert all(1e4 <= q.t_stop < 1e7 for q in qs)
    assert {q.grid for q in qs} == {0, 1, 2}
    # the draw is deterministic
    _, again = mixed_length_quenches()
    assert [(q.grid, q.t_stop) for q in qs] == [(q.grid, q.t_stop) for q in again]
    # log-uniform: the mean of log10(t_stop) sits near 5.5
    assert abs(sum(math.log10(q.t_stop) for q in qs) / 64 - 5.5) < 0.5
