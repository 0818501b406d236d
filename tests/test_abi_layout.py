"""The Python ctypes mirrors of the C ABI's structs have the C layout: size and
every field's offset, as a C compiler lays out include/pagani_gb300.h."""
import os
import shutil
import subprocess

import pytest

import gpuintegration_gb300 as pg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MIRRORS = {
    "pg_integrand": pg.PgIntegrand,
    "pg_result": pg.PgResult,
    "pg_options": pg.PgOptions,
    "pg_stats": pg.PgStats,
    "pg_mcubes_options": pg.PgMcubesOptions,
    "pg_iteration_record": pg.PgIterationRecord,
}


def _c_layout(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "pagani_gb300.h"', "int main(void) {"]
    for cname, mirror in MIRRORS.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in mirror._fields_:
            lines.append(f'  printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.check_call([cc, "-std=c99", "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    out = {}
    for line in subprocess.check_output([str(exe)], text=True).splitlines():
        cname, key, val = line.split()
        out[(cname, key)] = int(val)
    return out


def test_ctypes_mirrors_match_the_c_layout(tmp_path):
    c = _c_layout(tmp_path)
    for cname, mirror in MIRRORS.items():
        import ctypes
        assert ctypes.sizeof(mirror) == c[(cname, "size")], cname
        for field, _ in mirror._fields_:
            assert getattr(mirror, field).offset == c[(cname, field)], (cname, field)


def test_family_numbers_match_the_header(tmp_path):
    """The Python family constants are the C ABI's pg_family values, and every
    family has a name."""
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    names = {pg.CONSTANT: "CONSTANT", pg.OSCILLATORY: "OSCILLATORY", pg.PRODUCT_PEAK: "PRODUCT_PEAK",
             pg.CORNER_PEAK: "CORNER_PEAK", pg.GAUSSIAN: "GAUSSIAN", pg.C0: "C0", pg.DISCONTINUOUS: "DISCONTINUOUS",
             pg.PRODUCT: "PRODUCT", pg.NAN_VALUE: "NAN_VALUE", pg.BOX: "BOX", pg.FUN6: "FUN6",
             pg.GAUSSIAN_SUM: "GAUSSIAN_SUM"}
    lines = ['#include <stdio.h>', '#include "pagani_gb300.h"', "int main(void) {"]
    lines += [f'  printf("{n} %d\\n", (int)PG_FAMILY_{n});' for n in names.values()]
    lines += ['  printf("COUNT %d\\n", (int)PG_FAMILY_COUNT);', "  return 0;", "}"]
    src = tmp_path / "fam.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "fam"
    subprocess.check_call([cc, "-std=c99", "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = dict(line.split() for line in subprocess.check_output([str(exe)], text=True).splitlines())
    for value, n in names.items():
        assert int(got[n]) == value, n
    assert int(got["COUNT"]) == len(names) == len(pg.FAMILY_NAMES)
