"""The C-ABI library loads and exports every entry point include/*.h
declares (no GPU needed: nothing here launches a kernel)."""
import ctypes
import glob
import os
import re
import subprocess

import pphpc_gb300 as pp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(pp_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return names


def test_header_declares_core_api():
    names = declared_functions()
    for n in ("pp_load_params", "pp_stats_save", "pp_sim_create", "pp_sim_step",
              "pp_sim_destroy", "pp_batch_run", "pp_serve_create", "pp_serve_poll",
              "pp_radix_sort_host", "pp_move_host", "pp_cell_offsets_host"):
        assert n in names


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(pp.LIB_PATH)
    missing = [n for n in sorted(declared_functions()) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_mirror_covers_header():
    assert declared_functions() <= set(pp.ABI), declared_functions() - set(pp.ABI)


def test_nm_exports_are_c_symbols():
    out = subprocess.run(["nm", "-D", "--defined-only", pp.LIB_PATH],
                         stdout=subprocess.PIPE, text=True, check=True).stdout
    syms = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    for n in declared_functions():
        assert n in syms, n


def test_version_string():
    assert b"sm_103a" in pp.lib().pp_version()


def test_gpu_entry_fails_loudly_without_device():
    # Without a GPU, creating a simulation must fail with an error code;
    # there is no CPU fallback. (On a GPU host this returns success.)
    import ctypes as C
    p = pp.make_params(init_sheep=1, init_wolves=1, grid_x=4, grid_y=4, iters=1,
                       grass_restart=5, sheep_gain_from_food=4,
                       wolves_gain_from_food=20)
    h = C.c_void_p()
    rc = pp.lib().pp_sim_create(C.byref(p), 0, None, C.byref(h))
    if rc == pp.PP_SUCCESS:
        pp.lib().pp_sim_destroy(h)
    else:
        assert rc == pp.PP_ERR_CUDA


STATS_LAYOUT = [("sheep", 0), ("wolves", 4), ("grass", 8), ("sheep_en", 16),
                ("wolves_en", 24), ("grass_en", 32), ("errors", 40)]


def _c_layout(tmp_path, struct, fields):
    """sizeof/offsetof of `struct` as the C compiler lays it out from
    include/pphpc.h."""
    src = tmp_path / "layout.c"
    body = "".join('printf("%%zu\\n", offsetof(%s, %s));\n' % (struct, f)
                   for f in fields)
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "pphpc.h"\n'
                   'int main(void) {\nprintf("%%zu\\n", sizeof(%s));\n%s'
                   'return 0;\n}\n' % (struct, body))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"),
                    str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], stdout=subprocess.PIPE, text=True,
                         check=True).stdout.split()
    return int(out[0]), [int(x) for x in out[1:]]


def test_statistics_layout_matches_reference_order(tmp_path):
    # the reference's field order (pp_common.in.h:109-124: sheep, wolves,
    # grass, sheep_en, wolves_en, grass_en, errors) with 64-bit sums, in C
    # and in the Python mirror
    size, offs = _c_layout(tmp_path, "PPStatistics", [f for f, _ in STATS_LAYOUT])
    assert size == 48
    assert offs == [o for _, o in STATS_LAYOUT]
    assert ctypes.sizeof(pp.PPStatistics) == 48
    assert [f for f, _ in pp.PPStatistics._fields_] == [f for f, _ in STATS_LAYOUT]
    for f, o in STATS_LAYOUT:
        assert getattr(pp.PPStatistics, f).offset == o, f


def test_parameters_layout_matches_reference(tmp_path):
    # pp_common.in.h:129-157: thirteen unsigned ints in this order
    size, offs = _c_layout(tmp_path, "PPParameters", pp.PARAM_FIELDS)
    assert size == 4 * 13 == ctypes.sizeof(pp.PPParameters)
    assert offs == [4 * i for i in range(13)]
