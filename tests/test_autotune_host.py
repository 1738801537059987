"""Host side of the tile autotuner (no GPU): the wave-aware page candidates."""
import importlib


def test_wave_candidates():
    T = importlib.import_module("2018_7_vesicle_gb300.autotune")
    # 96^3 on 152 SMs x 4 resident blocks = 608 slots, 3 x 12 = 36 tiles per page set:
    # 6 pages -> 576 blocks (0.95 wave), 3 -> 1152 (1.89), 2 -> 1728 (2.84) fill their last
    # wave; 4 (864 blocks, 1.42 waves) and 5 (720, 1.18) do not, 4 stays as a default
    c = T.wave_candidates((96, 96, 96), sms=152)
    assert {2, 3, 6}.issubset(c) and 5 not in c and 7 not in c
    assert set(T.CANDIDATES).issubset(c)
    # a grid of many waves adds nothing below max_waves
    big = T.wave_candidates((256, 256, 256), sms=152)
    assert all(256 * -(-256 // k) / 608 <= 4.0 for k in set(big) - set(T.CANDIDATES))
    assert tuple(sorted(big)) == big
