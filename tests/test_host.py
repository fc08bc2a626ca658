"""Parameters file, validation and stats file (host code, no GPU)."""
import glob
import os

import numpy as np
import pytest

import pphpc_gb300 as pp

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
# the reference's configs directory, where the reference tree is present
REF_CONFIGS = os.path.join(os.environ.get("PPHPC_REFERENCE", "/root/reference"), "configs")


def test_load_golden_configs():
    p = pp.load_params(os.path.join(GOLDEN, "config100v1.txt"))
    assert (p.init_sheep, p.init_wolves, p.grid_x, p.grid_y, p.iters) == (400, 200, 100, 100, 4000)
    assert p.grid_xy == 10000
    p = pp.load_params(os.path.join(GOLDEN, "config400v2.txt"))
    assert (p.sheep_gain_from_food, p.sheep_reproduce_prob, p.grass_restart) == (30, 10, 15)
    p = pp.load_params(os.path.join(GOLDEN, "config12800v1.txt"))
    assert p.grid_xy == 163840000 and p.init_sheep == 6553600


@pytest.mark.skipif(not os.path.isdir(REF_CONFIGS), reason="reference tree not mounted")
def test_load_all_reference_configs():
    files = sorted(glob.glob(os.path.join(REF_CONFIGS, "*.txt")))
    assert len(files) == 20
    for f in files:
        p = pp.load_params(f)
        side = int(os.path.basename(f)[6:].split("v")[0])
        assert p.grid_x == side and p.grid_y == side
        assert pp.lib().pp_params_check(p, None, 0) == 0


def _write(tmp_path, text):
    f = tmp_path / "cfg.txt"
    f.write_text(text)
    return str(f)


GOOD = open(os.path.join(GOLDEN, "config100v1.txt")).read()


def test_missing_file(tmp_path):
    with pytest.raises(pp.PPError) as e:
        pp.load_params(str(tmp_path / "nope.txt"))
    assert e.value.code == pp.PP_UNABLE_TO_OPEN_PARAMS_FILE


@pytest.mark.parametrize("text", [
    GOOD.replace("GRID_X = 100\n", ""),                 # missing key
    GOOD + "GRID_X = 5\n",                              # repeated key
    GOOD.replace("ITERS", "ITERATIONS"),                 # unknown key
    GOOD.replace("GRID_Y = 100", "GRID_Y 100"),          # malformed record
    "",                                                  # empty
])
def test_invalid_files(tmp_path, text):
    with pytest.raises(pp.PPError) as e:
        pp.load_params(_write(tmp_path, text))
    assert e.value.code == pp.PP_INVALID_PARAMS_FILE


def test_whitespace_layout_is_free(tmp_path):
    # fscanf("%s = %d") semantics: records may be split across lines
    text = " ".join(GOOD.split())
    p = pp.load_params(_write(tmp_path, text))
    assert p.grid_x == 100 and p.iters == 4000


@pytest.mark.parametrize("field,value", [("grid_x", 0), ("grid_y", 70000),
                                         ("grass_restart", 0), ("grass_restart", 70000),
                                         ("sheep_reproduce_prob", 101)])
def test_params_check_limits(field, value):
    p = pp.load_params(os.path.join(GOLDEN, "config100v1.txt"))
    setattr(p, field, value)
    p.grid_xy = p.grid_x * p.grid_y
    assert pp.lib().pp_params_check(p, None, 0) == pp.PP_INVALID_ARGS


def _ref_row(s, cells):
    f32 = np.float32
    ms = f32(s[3]) / f32(s[0]) if s[0] else f32(0)
    mw = f32(s[4]) / f32(s[1]) if s[1] else f32(0)
    mg = f32(s[5]) / f32(cells)
    return "%d\t%d\t%d\t%f\t%f\t%f" % (s[0], s[1], s[2], ms, mw, mg)


def test_stats_format_matches_reference_printf():
    p = pp.load_params(os.path.join(GOLDEN, "config100v1.txt"))
    rows = np.load(os.path.join(GOLDEN, "stats_100v1_s0.npz"))["rows"]
    for r in rows[::97]:
        s = pp.PPStatistics(int(r[0]), int(r[1]), int(r[2]), int(r[3]), int(r[4]), int(r[5]))
        assert pp.format_row(s, p) == _ref_row([int(x) for x in r], 10000)


def test_stats_zero_counts():
    p = pp.load_params(os.path.join(GOLDEN, "config100v1.txt"))
    s = pp.PPStatistics(0, 0, 10000, 0, 0, 0, 0)
    assert pp.format_row(s, p) == "0\t0\t10000\t0.000000\t0.000000\t0.000000"


def test_stats_save(tmp_path):
    p = pp.load_params(os.path.join(GOLDEN, "config100v1.txt"))
    rows = np.load(os.path.join(GOLDEN, "stats_100v1_s0.npz"))["rows"][:11]
    st = [pp.PPStatistics(int(r[0]), int(r[1]), int(r[2]), int(r[3]), int(r[4]), int(r[5]))
          for r in rows]
    out = tmp_path / "stats.txt"
    pp.stats_save(str(out), st, p)
    lines = out.read_text().splitlines()
    assert len(lines) == 11
    assert lines[0] == _ref_row([int(x) for x in rows[0]], 10000)


def test_stats_save_unwritable(tmp_path):
    p = pp.load_params(os.path.join(GOLDEN, "config100v1.txt"))
    with pytest.raises(pp.PPError) as e:
        pp.stats_save(str(tmp_path / "no" / "dir" / "x.txt"), [pp.PPStatistics()], p)
    assert e.value.code == pp.PP_UNABLE_SAVE_STATS
