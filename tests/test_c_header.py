"""include/olgpu.h is a C header (the drop-in boundary is a C ABI): a C11
program that includes it builds with warnings as errors, links against
libolgpu.so and calls the entry points that need no GPU (version, defaults,
the host-only box plan, the server's configuration check, the argument check
of the cycle-event accessor)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(ROOT, "ollipticid_gb300", "_build")

PROGRAM = r"""
#include "olgpu.h"
#include <stdio.h>
#include <string.h>

int main(void)
{
  olgpu_problem p;
  olgpu_box_info boxes[64];
  int nb = 0, nl = 0, mg = 0;
  olgpu_server_config cfg;
  olgpu_server *s = NULL;
  printf("%s\n", olgpu_version());
  olgpu_problem_defaults(&p);
  p.equation = OLGPU_EQ_PUNCTURES;
  p.boundary = OLGPU_BC_ROBIN;
  p.method = OLGPU_METHOD_VCYCLE;
  p.numbh = 1;
  p.mp[0] = 0.5;
  p.n = 25;
  p.L = 40.0;
  p.order = 4;
  p.levels = 3;
  if (olgpu_plan_boxes(&p, boxes, 64, &nb, &nl, &mg) != OLGPU_OK) return 1;
  printf("boxes %d levels %d multigrid %d first %dx%dx%d\n", nb, nl, mg, boxes[0].nx, boxes[0].ny, boxes[0].nz);
  olgpu_server_config_defaults(&cfg);
  cfg.max_active = 0;
  if (olgpu_server_create(&cfg, &s) != OLGPU_ERR_INVALID_ARG) return 2;
  if (olgpu_cycle_events(NULL, 0, 0, NULL, NULL) != OLGPU_ERR_INVALID_ARG) return 4;
  p.order = 3;
  if (olgpu_plan_boxes(&p, boxes, 64, &nb, &nl, &mg) == OLGPU_OK) return 3;
  printf("refused: %s\n", olgpu_last_error());
  return 0;
}
"""


def test_header_is_c_and_the_library_links(tmp_path):
    from ollipticid_gb300 import build
    build.build()
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "abi_check.c"
    src.write_text(PROGRAM)
    exe = tmp_path / "abi_check"
    r = subprocess.run([cc, "-std=c11", "-Wall", "-Wextra", "-Werror", "-I", INCLUDE, str(src), "-o", str(exe),
                        "-L", BUILD, "-lolgpu", "-Wl,-rpath," + BUILD], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("olgpu ") and "boxes 4 levels 4 multigrid 1" in r.stdout
    assert "refused:" in r.stdout and "order" in r.stdout
