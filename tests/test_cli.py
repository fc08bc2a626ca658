"""Command-line drop-in (pp_gb300) error paths that need no GPU: the exit
status is the reference's pp_error_codes value (as an unsigned byte)."""
import os
import subprocess

import pphpc_gb300 as pp

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _run(*args):
    return subprocess.run([pp.CLI_PATH] + list(args), stdout=subprocess.PIPE,
                          stderr=subprocess.PIPE, text=True)


def test_missing_params_file(tmp_path):
    r = _run("-p", str(tmp_path / "missing.txt"))
    assert r.returncode == pp.PP_UNABLE_TO_OPEN_PARAMS_FILE & 0xff
    assert "Unable to open" in r.stderr


def test_invalid_params_file(tmp_path):
    f = tmp_path / "bad.txt"
    f.write_text("INIT_SHEEP = 1\n")
    r = _run("-p", str(f))
    assert r.returncode == pp.PP_INVALID_PARAMS_FILE & 0xff


def test_unknown_option():
    r = _run("--bogus")
    assert r.returncode == pp.PP_UNKNOWN_ARGS & 0xff


def test_non_option_argument():
    r = _run("extra")
    assert r.returncode == pp.PP_UNKNOWN_ARGS & 0xff


def test_invalid_limits(tmp_path):
    txt = open(os.path.join(GOLDEN, "config100v1.txt")).read().replace(
        "GRASS_RESTART = 10", "GRASS_RESTART = 0")
    f = tmp_path / "c.txt"
    f.write_text(txt)
    r = _run("-p", str(f))
    assert r.returncode == pp.PP_INVALID_ARGS & 0xff


def test_help():
    r = _run("-h")
    assert r.returncode == 0 and "Usage" in r.stderr
