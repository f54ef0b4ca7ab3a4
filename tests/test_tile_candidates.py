"""The order in which the library's tile tuner times its ten candidates
(a2c_gpp_autotune_tile: threads per site at 256-thread blocks, then the
pass-1 block at the best threads per site, then the pass-2 block at the
best of both; strictly faster replaces), decoded on the host."""
from a2c_gb300 import _tile_candidates


def test_candidates_follow_the_tuners_stages():
    ms = [5.0, 4.0, 4.5, 6.0,   # tps 1, 2, 4, 8 at 256/256: 2 wins
          3.9, 3.5, 3.7,        # pass-1 block 256, 512, 768 at tps 2: 512 wins
          3.6, 3.4, 3.45]       # pass-2 block 128, 256, 512
    tiles = [t for t, _ in _tile_candidates(ms)]
    assert tiles[:4] == [(1, 256, 256), (2, 256, 256), (4, 256, 256), (8, 256, 256)]
    assert tiles[4:7] == [(2, 256, 256), (2, 512, 256), (2, 768, 256)]
    assert tiles[7:] == [(2, 512, 128), (2, 512, 256), (2, 512, 512)]


def test_a_slower_stage_keeps_the_earlier_choice():
    ms = [5.0, 4.0, 4.5, 6.0, 4.1, 4.2, 4.3, 4.4, 4.0, 4.6]
    tiles = [t for t, _ in _tile_candidates(ms)]
    assert tiles[7:] == [(2, 256, 128), (2, 256, 256), (2, 256, 512)]
