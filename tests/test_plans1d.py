"""1D execution plans: the candidate list (qsg_candidate_plans_1d) is host
logic of libqsg.so, checked here without a GPU."""
import pytest

WALL = 1


@pytest.fixture(scope="module")
def q():
    import qusim_gb300 as q
    q.load()
    return q


def tuples(q, prec, n, boundary=0):
    return [p.as_tuple() for p in q.candidate_plans_1d(prec, n, boundary)]


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_four_step_splits(q, prec):
    for lg in range(13, 24):
        n = 1 << lg
        plans = tuples(q, prec, n)
        fs = [p for p in plans if p[0] == 1]
        assert fs, n
        # the default split first among the four-step plans: n1 = n2 or 2 n2, but
        # 4096 x 1024 rather than 2048 x 2048 (columns of 2048 run two per CTA)
        n1 = fs[0][1]
        assert (n1 * n1 in (n, 2 * n) or (n1 == 4096 and n // n1 == 1024)) and fs[0][2] == 0
        assert n < (1 << 22) or n // n1 <= 2048 and (n > (1 << 22) or n // n1 == 1024)
        for kind, n1, tma in fs:
            n2 = n // n1
            assert n1 * n2 == n and 64 <= n1 <= 4096 and 64 <= n2 <= 2048
            # tensor-copy column passes: complex64, columns of 128 .. 512
            assert not tma or (prec == "mixed" and n2 in (128, 256, 512))
        assert len(set(plans)) == len(plans)


def test_resident_plans(q):
    assert tuples(q, "mixed", 1024) == [(0, 0, 0)]
    assert tuples(q, "mixed", 8192)[0] == (0, 0, 0)   # one CTA where it fits: the default
    assert (0, 0, 0) not in tuples(q, "fp64", 8192)  # complex128 holds 4096 in one CTA
    assert tuples(q, "fp64", 4096) == [(0, 0, 0)]


def test_lengths_without_choices(q):
    # Bluestein lengths: one plan; lengths beyond every plan: none
    assert tuples(q, "mixed", 1000) == [(0, 0, 0)]
    assert tuples(q, "fp64", 4095) == [(0, 0, 0)]
    # longer lengths that are not powers of two: Bluestein on the four-step passes
    # of the smallest power of two M >= 2n - 1, its default split
    assert tuples(q, "mixed", 5000) == [(1, 128, 0)]      # M = 16384
    assert tuples(q, "fp64", 4097) == [(1, 128, 0)]
    assert tuples(q, "mixed", 100000) == [(1, 512, 0)]    # M = 262144
    assert tuples(q, "fp64", 131071) == [(1, 512, 0)]
    assert tuples(q, "mixed", 131073) == [(1, 1024, 0)]   # M = 524288
    assert tuples(q, "fp64", 524287) == [(1, 1024, 0)]    # M = 1048576
    assert tuples(q, "mixed", 2097151) == [(1, 4096, 0)]  # M = 4194304
    assert tuples(q, "fp64", 4194303) == [(1, 4096, 0)]   # M = 8388608
    assert tuples(q, "mixed", 4194305) == []              # M = 2^24: beyond the passes
    assert tuples(q, "mixed", 1 << 24) == []
    assert tuples(q, "mixed", 32) == [(0, 0, 0)]   # powers of two below 64: Bluestein
    assert tuples(q, "mixed", 1) == []
    assert tuples(q, 7, 1024) == []                # unknown precision


def test_wall_plans(q):
    # one CTA holds the 2n extension up to n = 4096 (complex64); above, the
    # four-step plans of the periodic 2n extension, without tensor copies
    assert tuples(q, "mixed", 4096, WALL) == [(0, 0, 0)]
    plans = tuples(q, "mixed", 65536, WALL)
    assert plans and all(k == 1 and t == 0 for k, _, t in plans)
    assert {n1 for _, n1, _ in plans} == {n1 for k, n1, _ in tuples(q, "mixed", 131072) if k == 1}
    assert tuples(q, "mixed", 524288, WALL)[0] == (1, 1024, 0)   # the 2^20 extension
    assert tuples(q, "mixed", 1 << 21, WALL)[0] == (1, 4096, 0)  # the 2^22 extension
    assert tuples(q, "mixed", 1 << 22, WALL)[0] == (1, 4096, 0)  # the 2^23 extension
    assert tuples(q, "mixed", 1 << 23, WALL) == []
    # any other length: one Bluestein kernel on the 2n extension (2n - 1 <= 8192 / 4096)
    assert tuples(q, "mixed", 1000, WALL) == [(0, 0, 0)]
    assert tuples(q, "mixed", 32, WALL) == [(0, 0, 0)]
    assert tuples(q, "mixed", 2048, WALL) == [(0, 0, 0)]
    assert tuples(q, "fp64", 1500, WALL) == [(0, 0, 0)]
    # longer: Bluestein on the four-step passes of M >= 4n - 1 (the extension's 2 (2n) - 1)
    assert tuples(q, "mixed", 3000, WALL) == [(1, 128, 0)]     # M = 16384
    assert tuples(q, "fp64", 3000, WALL) == [(1, 128, 0)]
    assert tuples(q, "mixed", 65535, WALL) == [(1, 512, 0)]    # M = 262144
    assert tuples(q, "fp64", 262143, WALL) == [(1, 1024, 0)]   # M = 1048576
    assert tuples(q, "fp64", 1048575, WALL) == [(1, 4096, 0)]  # M = 4194304
    assert tuples(q, "fp64", 2097151, WALL) == [(1, 4096, 0)]  # M = 8388608
    assert tuples(q, "mixed", 2097153, WALL) == []
    assert tuples(q, "mixed", 1, WALL) == []
