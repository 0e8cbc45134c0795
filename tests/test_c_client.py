"""The C-ABI from a plain C99 client (no Python, no C++): the header compiles as C99 with
-pedantic, and a C program links the library dynamically, resolves entry points and calls
ufe_init (UFE_OK on an sm_103a device, UFE_NO_DEVICE elsewhere)."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

from ufemism_gb300 import _native as nat

C_SOURCE = r"""
#include <stdio.h>
#include <dlfcn.h>
#include "ufemism_gb300.h"
int main(int argc, char **argv) {
  void *h = dlopen(argv[1], RTLD_NOW);
  if (!h) { printf("dlopen failed\n"); return 2; }
  int (*init)(int) = (int (*)(int))dlsym(h, "ufe_init");
  int (*solve)(ufe_mesh_h, const ufe_params *, const ufe_ssa_in *, ufe_ssa_inout *, ufe_ssa_out *,
               ufe_ssa_stats *) = (int (*)(ufe_mesh_h, const ufe_params *, const ufe_ssa_in *, ufe_ssa_inout *,
                                            ufe_ssa_out *, ufe_ssa_stats *))dlsym(h, "ufe_ssa_solve");
  if (!init || !solve) { printf("missing symbol\n"); return 3; }
  ufe_params p = {0};
  /* argument validation needs no device */
  if (solve(NULL, &p, NULL, NULL, NULL, NULL) != UFE_BAD_ARG) return 4;
  printf("%d\n", init(0));
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_c99_client_links_and_calls(tmp_path):
    lib = nat.lib_path()
    if not os.path.exists(lib):
        nat.load()
    inc = os.path.join(ROOT, "include")
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-fsyntax-only", "-x", "c",
                    os.path.join(inc, "ufemism_gb300.h")], check=True)
    src = tmp_path / "client.c"
    src.write_text(C_SOURCE)
    exe = tmp_path / "client"
    subprocess.run(["gcc", "-std=c99", "-I", inc, str(src), "-o", str(exe), "-ldl"], check=True)
    out = subprocess.run([str(exe), lib], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert int(out.stdout.strip().splitlines()[-1]) in (nat.UFE_OK, nat.UFE_NO_DEVICE)
