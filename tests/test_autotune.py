"""Host logic of the contraction autotuner (no GPU): the choice per class with its tie margin,
and the merging of adjacent classes that chose the same schedule."""
from manifoldem_python_gb300 import autotune as A


def test_pick_prefers_the_simplest_schedule_within_the_margin():
    base = A.CANDIDATES[0]
    ms = {c: 1.0 for c in A.CANDIDATES}
    assert A.pick(ms) == base                          # ties: the first (simplest) candidate
    ms[A.CANDIDATES[3]] = 0.985                        # 1.5% faster: inside the margin
    assert A.pick(ms) == base
    ms[A.CANDIDATES[3]] = 0.90                         # 10% faster: chosen
    assert A.pick(ms) == A.CANDIDATES[3]
    ms[A.CANDIDATES[4]] = 0.89                         # 1% faster again: kept the earlier one
    assert A.pick(ms) == A.CANDIDATES[3]


def test_adjacent_equal_classes_merge_into_one_launch():
    mk = lambda n, tn, p=0: dict(max_n=n, persistent=p, accumulators=2, tile_n=tn, tile_m=128,
                                 rep_n=n // 2, ms={})
    big = 2 ** 31 - 1
    out = A.merge_classes([mk(192, 128), mk(640, 256), mk(1536, 256), mk(big, 256, 1)])
    assert [(c['max_n'], c['tile_n'], c['persistent']) for c in out] == \
        [(192, 128, 0), (1536, 256, 0), (big, 256, 1)]
    assert len(out[1]['merged']) == 2
    arr = A.to_c(out)
    assert [arr[i].max_n for i in range(3)] == [192, 1536, big]
    assert arr[1].tile_n == 256 and arr[2].persistent == 1 and arr[0].tile_m == 128
