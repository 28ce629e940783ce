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


LAYOUT = r"""
#include "olgpu.h"
#include <stddef.h>
#include <stdio.h>
#define S(t) printf(#t " %zu\n", sizeof(t))
#define O(t, f) printf(#t "." #f " %zu\n", offsetof(t, f))
int main(void)
{
  S(olgpu_problem); S(olgpu_box_info); S(olgpu_stop_rule); S(olgpu_report); S(olgpu_cycle_event);
  S(olgpu_server_config); S(olgpu_server_result); S(olgpu_box_fields);
  O(olgpu_stop_rule, du_tol); O(olgpu_report, final_du); O(olgpu_report, final_part); O(olgpu_server_config, du_tol);
  O(olgpu_server_result, final_du); O(olgpu_problem, method); O(olgpu_server_config, batch_max);
  O(olgpu_server_config, batch_window);
  return 0;
}
"""


def test_ctypes_mirror_has_the_header_layout(tmp_path):
    """Every struct of the ABI has the same size and field offsets in the C
    header and in the Python mirror (ollipticid_gb300/_abi.py)."""
    import ctypes as C
    from ollipticid_gb300 import _abi
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "layout.c"
    src.write_text(LAYOUT)
    exe = tmp_path / "layout"
    r = subprocess.run([cc, "-std=c11", "-I", INCLUDE, str(src), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = dict(line.rsplit(" ", 1) for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                               check=True).stdout.splitlines())
    mirror = {"olgpu_problem": _abi.Problem, "olgpu_box_info": _abi.BoxInfo, "olgpu_stop_rule": _abi.StopRule,
              "olgpu_report": _abi.Report, "olgpu_cycle_event": _abi.CycleEvent,
              "olgpu_server_config": _abi.ServerConfig, "olgpu_server_result": _abi.ServerResult,
              "olgpu_box_fields": _abi.BoxFields}
    for name, cls in mirror.items():
        assert int(got[name]) == C.sizeof(cls), name
    for key, val in got.items():
        if "." in key:
            t, f = key.split(".")
            assert int(val) == getattr(mirror[t], f).offset, key
