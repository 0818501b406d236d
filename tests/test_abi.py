"""C ABI: the library loads without a GPU and exports what include/pagani_gb300.h declares."""
import ctypes

import gpuintegration_gb300 as pg


def test_every_declared_symbol_is_exported(lib):
    names = pg.declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_options_default_matches_reference(lib):
    o = pg.default_options()
    assert o.relerr_classification == 1          # Workspace.cuh:360-368
    assert o.max_iters == 700                    # Workspace.cuh:399
    assert o.device_mem_model == 16e9            # heuristic_classifier.cuh:89-94


def test_feval_formula(lib):
    expect = {2: 33, 3: 77, 4: 153, 5: 273, 6: 453, 7: 717, 8: 1105, 9: 1689, 10: 2605}
    for d, fe in expect.items():
        assert lib.pg_feval(d) == fe
    assert lib.pg_feval(1) == -1


def test_struct_sizes_match_header(lib):
    assert ctypes.sizeof(pg.PgIntegrand) == 8 + 16 * 8 * 2 + 8
    assert ctypes.sizeof(pg.PgResult) == 3 * 8 + 4 * 8 + 2 * 4
