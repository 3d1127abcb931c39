"""The C-ABI from a plain C caller: include/flint_gpu.h compiles as strict C99
(-pedantic -Werror), and a C program linked against the library runs the
host-only entry points (version, IR blob parsing, table-file reading) and gets
their status codes and error texts.  Host only: no GPU."""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

C_SRC = r"""
#include <stdio.h>
#include <string.h>
#include "flint_gpu.h"

int main(int argc, char** argv) {
  flint_ir_t ir = NULL;
  flint_table_set_t ts = NULL;
  flint_mech_desc d;
  FILE* f;
  static unsigned char blob[1 << 20];
  size_t nb;
  int rc;
  if (argc < 3) return 2;
  if (!flint_version() || !flint_version()[0]) return 3;
  /* a valid blob parses and describes its mechanism */
  f = fopen(argv[1], "rb");
  if (!f) return 4;
  nb = fread(blob, 1, sizeof blob, f);
  fclose(f);
  rc = flint_ir_parse(blob, (int64_t)nb, &ir);
  if (rc != FLINT_OK) { printf("parse %d %s\n", rc, flint_last_error()); return 5; }
  if (flint_ir_desc(ir, &d) != FLINT_OK) return 6;
  if (flint_ir_bytes(d.ns, d.nr, d.nasa9 != NULL) != (int64_t)nb) return 7;
  printf("ns=%d nr=%d r_eos=%.2f\n", d.ns, d.nr, d.r_eos);
  flint_ir_free(ir);
  /* a truncated blob is refused with a reason */
  rc = flint_ir_parse(blob, (int64_t)nb - 8, &ir);
  if (rc != FLINT_ERR_ARG || ir != NULL || !strstr(flint_last_error(), "bytes")) return 8;
  /* a folder without FLINT's files is an I/O error */
  rc = flint_tables_read(argv[2], NULL, &ts);
  if (rc != FLINT_ERR_IO || ts != NULL || !strstr(flint_last_error(), "phase.txt")) return 9;
  printf("ok\n");
  return 0;
}
"""


def test_c_caller(tmp_path):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    from flint_gb300 import mechgen, native
    if not os.path.exists(native.LIB_PATH):
        from flint_gb300 import build
        build.build_all()
    src = tmp_path / "caller.c"
    src.write_text(C_SRC)
    exe = tmp_path / "caller"
    libdir = os.path.dirname(native.LIB_PATH)
    libname = os.path.basename(native.LIB_PATH)[3:-3]          # libNAME.so -> NAME
    r = subprocess.run([gcc, "-std=c99", "-pedantic", "-Wall", "-Wextra", "-Werror", "-I",
                        os.path.join(REPO, "include"), str(src), "-L", libdir, "-l" + libname,
                        "-Wl,-rpath," + libdir, "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    blob = tmp_path / "c2.flir"
    m = mechgen.load("c2")
    blob.write_bytes(m.to_ir())
    empty = tmp_path / "empty"
    empty.mkdir()
    r = subprocess.run([str(exe), str(blob), str(empty)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert f"ns={m.ns} nr={m.nr}" in r.stdout and r.stdout.strip().endswith("ok")
