"""2D execution plans: which power-of-two grids have split-k plans
(qsg_candidate_plans, host logic of libqsg.so), checked without a GPU."""
import pytest


@pytest.fixture(scope="module")
def lib():
    import qusim_gb300 as q
    return q._lib.load()


MIXED, FP64 = 1, 0


def count(lib, prec, nx, ny):
    return lib.qsg_candidate_plans(prec, nx, ny, None, 0)


def test_square_grids_up_to_4096(lib):
    for side in (128, 256, 512, 1024, 2048, 4096):
        assert count(lib, MIXED, side, side) > 0, side
        assert count(lib, FP64, side, side) > 0, side


def test_one_side_of_8192(lib):
    # columns of 8192 (x): the x split G = 4 leaves 2048-point column transforms
    for ny in (128, 1024, 4096):
        assert count(lib, MIXED, 8192, ny) > 0, ny
    for ny in (128, 2048):
        assert count(lib, FP64, 8192, ny) > 0, ny
    assert count(lib, FP64, 8192, 4096) == 0        # 4 complex128 rows of 4096: 256 KB
    # rows of 8192 (y): one or two rows per row-pass unit, complex64 only
    for nx in (128, 1024, 4096):
        assert count(lib, MIXED, nx, 8192) > 0, nx
        assert count(lib, FP64, nx, 8192) == 0, nx
    assert count(lib, MIXED, 8192, 8192) == 0       # needs G = 4 with 8192-point rows


def test_no_plans_outside_the_powers_of_two(lib):
    assert count(lib, MIXED, 1000, 1024) == 0       # Bluestein passes instead
    assert count(lib, MIXED, 64, 1024) == 0
    assert count(lib, MIXED, 16384, 256) == 0
    assert count(lib, 7, 1024, 1024) == 0           # unknown precision
