"""The library's host tile planner (ustb_plan_tiles_host, used by ustb_plan_create)
against the Python planner of fast.py (plan_tiles, order_by_cost, refine_tiles):
the same tile maps, lane for lane, without a GPU."""
import numpy as np
import pytest

import bench
from ustb_gb300 import fast, synth
from ustb_gb300.enums import Window
from ustb_gb300.geometry import Apodization
from ustb_gb300.plan import library_tiles
from ustb_gb300.uff import LinearScan, Point, Probe, Scan, Wave


@pytest.mark.parametrize("kind", ["iq_cpwc", "dw_sector", "rf_plane_wave", "sta", "matrix_3d"])
def test_library_planner_matches_python_planner(kind):
    wl = synth.CONFIGS[kind](device="cpu", scale=0.3 if kind != "matrix_3d" else 0.25)
    g = bench.build_das(wl).fast_geometry("cpu")
    lt = library_tiles(g)
    assert lt.shape == g.tiles.shape
    assert np.array_equal(lt, g.tiles)


def test_library_planner_splits_by_tabulated_delays():
    probe = Probe.linear_array(16, 0.3e-3)
    scan = LinearScan(np.linspace(-3e-3, 3e-3, 48), np.linspace(5e-3, 14e-3, 96))
    seq = [Wave(source=Point.from_xyz(x, 0, 9e-3)) for x in (-1e-3, 0.0, 1e-3)]
    g = fast.FastGeometry(probe, scan, seq, 20e6, 0.0, 5e6, 1540.0, "cpu", Apodization(window=Window.boxcar))
    assert g.d_txdelay is not None
    lt = library_tiles(g)
    assert np.array_equal(np.sort(lt[lt >= 0]), np.arange(scan.N_pixels))
    # the same pixel sets as the Python refinement (both halve the same lists)
    key = lambda t: sorted(tuple(sorted(r[r >= 0])) for r in t)
    assert key(lt) == key(g.tiles)


def test_library_planner_on_a_pixel_list():
    rng = np.random.default_rng(3)
    P = 5000
    scan = Scan(rng.uniform(-5e-3, 5e-3, P), np.zeros(P), rng.uniform(5e-3, 25e-3, P))
    g = fast.FastGeometry(Probe.linear_array(32, 0.3e-3), scan, [Wave.plane(0.0)], 20e6, 0.0, 5e6, 1540.0, "cpu",
                          Apodization(window=Window.tukey25, f_number=1.5))
    lt = library_tiles(g)
    assert np.array_equal(np.sort(lt[lt >= 0]), np.arange(P))  # every pixel once
    assert np.all(lt[:, 0] >= 0)                                 # lane 0 of every tile live
    limit = fast.SPAN_LIMIT * 1540.0 / 20e6
    for row in lt:
        b = scan.xyz[row[row >= 0]]
        assert len(b) == 1 or np.linalg.norm(b.max(0) - b.min(0)) <= limit * (1 + 1e-9)


@pytest.mark.parametrize("what", ["pixel", "element"])
def test_library_planner_rejects_non_finite_positions(what):
    import ctypes

    from ustb_gb300 import _lib
    from ustb_gb300.enums import Precision
    from ustb_gb300.plan import plan_desc

    wl = synth.CONFIGS["iq_cpwc"](device="cpu", scale=0.1)
    g = bench.build_das(wl).fast_geometry("cpu")
    d, keep = plan_desc(g, 1024, Precision.fp32, True)
    ptr = d.geometry.pixel_xyz if what == "pixel" else d.geometry.element_xyz
    ctypes.cast(ptr, ctypes.POINTER(ctypes.c_float))[4] = float("nan")
    n = int(_lib.lib().ustb_plan_tiles_host(ctypes.addressof(d), None, 0))
    assert n == -1  # USTB_E_ARG
    assert b"non-finite" in _lib.lib().ustb_last_error()


def test_ctas_per_tile_range():
    """dimension.both runs 1 to 4 CTAs per tile (0: the library's choice); more is refused."""
    scan = LinearScan(np.linspace(-2e-3, 2e-3, 16), np.linspace(5e-3, 9e-3, 32))
    args = (Probe.linear_array(32, 0.3e-3), scan, [Wave.plane(0.0)], 20e6, 0.0, 5e6, 1540.0, "cpu",
            Apodization(window=Window.boxcar))
    for c in range(5):
        assert fast.FastGeometry(*args, ctas_per_tile=c).c.ctas_per_tile == c
    with pytest.raises(ValueError):
        fast.FastGeometry(*args, ctas_per_tile=5)
