"""The work model the rooflines divide by (perf/work_model.py): its constants, and that
bench.py reports with exactly these (no second copy of a constant)."""
import pytest

from perf import work_model as wm


def test_pair_and_kspace_constants():
    assert wm.FLOP_PAIR_LJ == 29.0 and wm.FLOP_PAIR_ELEC == 42.0
    assert wm.FLOP_PAIR == 55.0  # LJ + electrostatics share the distance and the accumulation
    assert (wm.FLOP_K_S, wm.FLOP_K_F) == (10.0, 12.0)
    assert wm.SF_BYTES_PER_SITE == 64 * 4


def test_byte_models():
    # one full-list entry pair (two entries, one evaluated): 2 x 20 B + 8 slots x 32 B; one site 40 B
    assert wm.neighbour_streaming_bytes(2, 1) == pytest.approx(2 * 20 + 8 * 32 + 40)
    assert wm.list_build_bytes(1, 1) == pytest.approx(24 + 72)


def test_bench_uses_the_model():
    import bench
    for name in ("FLOP_PAIR", "FLOP_K_S", "FLOP_K_F", "FLOP_SK_ROWKZ", "FLOP_SK_ROW", "FLOP_KF_ROWKZ",
                 "FLOP_KF_ROW", "SF_BYTES_PER_SITE", "neighbour_streaming_bytes", "list_build_bytes"):
        assert getattr(bench, name) is getattr(wm, name)
