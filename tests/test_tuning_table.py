"""The committed tuning table (cubigfloat_gb300/tuned_configs.txt, loaded by the library at
start-up): every (operation, limb count) from 1 to 512 is covered exactly once, by a
configuration that exists, runs that operation and holds that many limbs; and the table
survives a read / write round trip of cubigfloat_gb300.tune."""
import os

from cubigfloat_gb300 import tune

# (lanes, tile limbs, block pairs) per configuration, as in csrc/fpa_launch.h
SHAPES = [(4, 2, 1), (8, 2, 1), (8, 4, 1), (16, 4, 1), (32, 4, 1), (32, 8, 1), (32, 16, 1), (16, 8, 1),
          (8, 16, 1), (16, 16, 1), (8, 4, 2), (8, 4, 4), (16, 4, 2), (8, 8, 4), (16, 8, 2), (4, 4, 8),
          (4, 8, 1), (4, 16, 1), (1, 8, 16), (1, 8, 8)]


def supports(cfg, op):
    if cfg >= 18:                      # one thread per operation: mul, div and sqrt
        return op in (2, 3, 4)
    return cfg < 16 or op <= 1 or (cfg == 16 and op == 2)


def test_table_covers_every_size_once_with_a_valid_configuration():
    rows = tune.read()
    seen = {}
    for op, lo, hi, cfg, _ in rows:
        assert 0 <= op <= 4 and 1 <= lo <= hi <= 512 and 0 <= cfg < len(SHAPES), (op, lo, hi, cfg)
        g, k, r = SHAPES[cfg]
        assert g * k * r >= hi, f"configuration {cfg} cannot hold {hi} limbs"
        assert supports(cfg, op), f"configuration {cfg} does not run op {op}"
        for n in range(lo, hi + 1):
            assert (op, n) not in seen, f"op {op} limbs {n} listed twice"
            seen[(op, n)] = cfg
    for op in range(5):
        for n in range(1, 513):
            assert (op, n) in seen, f"op {op} limbs {n} missing"


def test_table_round_trip(tmp_path):
    rows = tune.read()
    out = os.path.join(tmp_path, "t.txt")
    tune.write(rows, out)
    again = tune.read(out)
    assert [r[:4] for r in again] == [r[:4] for r in sorted(rows, key=lambda r: (r[0], r[1]))]


def test_shapes_match_the_library():
    import cubigfloat_gb300 as fpa
    assert fpa.configs() == SHAPES
