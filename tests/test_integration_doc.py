"""The C examples of the integration guide compile against include/*.h (gcc -fsyntax-only), with
PETSc's names stubbed, so the documented calls keep matching the headers."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PRELUDE = r"""
#include <stddef.h>
typedef int PetscErrorCode;
typedef struct _p_Vec *Vec;
#define PETSC_COMM_SELF 0
#define PETSC_ERR_LIB 76
#define SETERRQ(comm, code, msg) return (code)
#define PetscMin(a, b) ((a) < (b) ? (a) : (b))
static void VecGetArrayRead(Vec v, const double **a) { (void)v; *a = NULL; }
static void VecGetArray(Vec v, double **a) { (void)v; *a = NULL; }
static void VecRestoreArray(Vec v, double **a) { (void)v; (void)a; }
static void VecRestoreArrayRead(Vec v, const double **a) { (void)v; (void)a; }
/* the caller's variables the examples use */
static int mx, my, p, nrecv, stf_type[2], rows, shot;
static double vp, vs, rho, time_max, src_xy[4], src_m[8], stf_par[6], xr_list[2], time_;
static double times[100], stf_buf[200], trace_buf[101 * 7];
static double *LA_u, *LA_v, *LA_a, *u_, *v_, *a_;
static long k, n;
static Vec u, F;
static se2gpu_solver *h;
#define time time_
#define stf stf_buf
#define traces trace_buf
"""


def c_blocks():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    return re.findall(r"```c\n(.*?)```", text, re.S)


def test_integration_guide_c_examples_compile(tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    blocks = c_blocks()
    assert len(blocks) >= 3
    includes, bodies = [], []
    for i, b in enumerate(blocks):
        inc = [ln for ln in b.splitlines() if ln.startswith("#include")]
        includes += inc
        body = "\n".join(ln for ln in b.splitlines() if not ln.startswith("#include"))
        if i == 1:     # the second example takes the caller's const view of u
            body = body.replace("LA_u", "LA_uc")
            body = "const double *LA_uc; double *LA_F;\n" + body
        if i == 2:
            body = body.replace("u, v, a)", "u_, v_, a_)")
        bodies.append(f"static PetscErrorCode example_{i}(void)\n{{\n{body}\nreturn 0;\n}}\n")
    src = ('#include "se2host.h"\n#include "se2gpu.h"\n' + PRELUDE + "\n".join(bodies))
    assert '#include "se2host.h"' in includes and '#include "se2gpu.h"' in includes
    f = tmp_path / "integration_examples.c"
    f.write_text(src)
    r = subprocess.run(["gcc", "-std=c99", "-fsyntax-only", "-Wall", "-Wno-unused-function",
                        "-Werror=implicit-function-declaration", "-Werror=incompatible-pointer-types",
                        "-Werror=int-conversion",
                        "-I", os.path.join(ROOT, "include"), str(f)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
