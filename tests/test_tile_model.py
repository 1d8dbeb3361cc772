"""CPU: the launch model behind the compensated form's default r-chunk
(csrc/mwsep_host.cu static_tile_cost / model_kchunk, exported as
mwsep_model_tile_cost / mwsep_model_kchunk), against a numpy restatement of
the same model (tile by tile, warp by warp) and the choices it made on the
GB300 measurements: 70 r-bins for the full-size wedge (1600 x 640 x 140,
convolve 120, 3 streams), where a sweep of 28 / 32 / 35 / 47 / 70 / 140 bins
timed 17.3 / 16.3 / 16.6 / 16.6 / 16.0 / 16.2 ms with a fixed share of
tiles per warp."""
import ctypes as C

import numpy as np
import pytest

SMS, BPS, WPB, GROUP = 152, 2, 8, 256  # GB300, 2 blocks of 8 warps, 8 points x 32 lanes per group


def _restated_cost(R, Cv, group, nmb, nnu, kc, p, sms=SMS, bps=BPS, wpb=WPB):
    nk = (R + kc - 1) // kc
    W = sms * bps * wpb
    tiles = nmb * nnu * nk
    chunk_cost = np.array([-(-min(kc, R - k * kc) * Cv // group) + p for k in range(nk)], float)
    wt = np.arange(tiles)
    sm = ((wt % W) // wpb) % sms
    return np.bincount(sm, weights=chunk_cost[wt // (nmb * nnu)], minlength=sms).max()


@pytest.fixture(scope="module")
def lib(built_library):
    from milkywayathome_client_gb300 import native as N
    return N.lib()


@pytest.mark.parametrize("kc", [28, 32, 35, 47, 70, 140])
def test_cost_matches_restatement(lib, kc):
    nmb, nnu = 1600 // 32, 640
    got = lib.mwsep_model_tile_cost(140, 120, GROUP, nmb * nnu, kc, SMS, BPS, WPB, 0.5)
    assert got == pytest.approx(_restated_cost(140, 120, GROUP, nmb, nnu, kc, 0.5), rel=1e-12)


def test_ragged_wedge_cost(lib):
    # a wedge whose mu columns do not fill the last tile and whose r range is not a chunk multiple
    nmb, nnu = (333 + 31) // 32, 77
    for kc in (9, 17, 50):
        got = lib.mwsep_model_tile_cost(50, 30, GROUP, nmb * nnu, kc, SMS, BPS, WPB, 0.5)
        assert got == pytest.approx(_restated_cost(50, 30, GROUP, nmb, nnu, kc, 0.5), rel=1e-12)


def _choice(lib, R, Cv, S, mu, nu):
    k, cost = C.c_int(), C.c_double()
    assert lib.mwsep_model_kchunk(R, Cv, S, mu, nu, SMS, BPS, C.byref(k), C.byref(cost)) == 0
    return k.value, cost.value


def test_full_size_choice(lib):
    k, cost = _choice(lib, 140, 120, 3, 1600, 640)
    assert k == 70
    # the cheapest of every chunk from the four-group floor (32 bins here) up
    costs = {kc: _restated_cost(140, 120, GROUP, 50, 640, kc, 0.5) for kc in range(32, 141)}
    assert cost == pytest.approx(min(costs.values()), rel=1e-12)
    assert min(costs, key=costs.get) == 70


def test_choices_of_other_wedges(lib):
    assert _choice(lib, 140, 60, 3, 400, 160)[0] == 140   # 400 x 160 x 140, convolve 60
    assert _choice(lib, 70, 30, 1, 200, 80)[0] == 70      # a small wedge: one chunk


def test_invalid_input(lib):
    assert lib.mwsep_model_tile_cost(0, 120, GROUP, 10, 5, SMS, BPS, WPB, 0.5) == -1.0
    k = C.c_int()
    assert lib.mwsep_model_kchunk(140, 120, 9, 1600, 640, SMS, BPS, C.byref(k), None) != 0
