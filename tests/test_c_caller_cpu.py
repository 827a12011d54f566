"""The drop-in boundary from a plain C caller: a C99 program that includes
include/sepx.h compiles, links against the built library and gets an error
status with a message back (no GPU needed: the call fails on its NULL
buffer before any device work)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

PROG = r"""
#include <stdio.h>
#include <string.h>
#include "sepx.h"
#include "sepx_ops.h"
#include "sepx_sepio.h"

int main(void) {
  int rc = sepx_transfer_vel_func1(4, 4, 4, NULL);
  const char *msg = sepx_last_error();
  printf("%d %s\n", rc, msg);
  if (rc == 0 || strstr(msg, "NULL") == NULL) return 1;
  rc = sepx_rtm_op_forward(NULL, 0, NULL, NULL);
  if (rc == 0) return 2;
  return 0;
}
"""


def test_c99_program_links_and_gets_errors(tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("no gcc")
    from sep_code_gb300 import build
    from sep_code_gb300._lib import lib  # noqa: F401  (builds the library if needed)
    src = tmp_path / "caller.c"
    src.write_text(PROG)
    exe = tmp_path / "caller"
    libdir = build.LIB.parent
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", str(src), f"-I{ROOT / 'include'}",
                    f"-L{libdir}", "-lsepx", f"-Wl,-rpath,{libdir}", "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert "NULL" in r.stdout
