"""The C ABI from C: a C99 program includes include/kymatio_gb300.h, links
the library and drives the host-side entry points (version, plan geometry,
launch groups, argument errors).  No device work, so it runs without a GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r'''
#include <stdio.h>
#include <string.h>
#include "kymatio_gb300.h"

int main(void) {
  kym_s2d_plan* plan = NULL;
  int Mp, Np, C, orr, occ, nf, g, level, ntasks, rows, cols, fold, cluster;
  if (kym_s2d_plan_create(256, 256, 3, 8, 2, 0, &plan) != KYM_OK) return 1;
  if (kym_s2d_plan_info(plan, &Mp, &Np, &C, &orr, &occ, &nf) != KYM_OK) return 2;
  printf("version %s\n", kym_version());
  printf("padded %d %d channels %d out %d %d filters %d\n", Mp, Np, C, orr, occ, nf);
  for (g = 0; g < kym_s2d_group_count(plan); ++g) {
    if (kym_s2d_group_info(plan, g, &level, &ntasks, &rows, &cols, &fold, &cluster) != KYM_OK) return 3;
    printf("group %d level %d tasks %d size %dx%d fold %d\n", g, level, ntasks, rows, cols, fold);
  }
  if (kym_s2d_forward(plan, NULL, NULL, 1, NULL, 0, NULL, 0, NULL) != KYM_ERR_INVALID) return 4;
  if (kym_s2d_plan_destroy(plan) != KYM_OK) return 5;
  return 0;
}
'''


def test_header_and_library_from_c(tmp_path):
    from kymatio_gb300 import _lib
    lib = _lib.lib_path()
    if not os.path.exists(lib):
        _lib.load(build_if_missing=True)
    cc = shutil.which('gcc') or shutil.which('cc')
    if cc is None:
        pytest.skip('no C compiler')
    src = tmp_path / 'abi.c'
    src.write_text(PROGRAM)
    exe = tmp_path / 'abi'
    libdir = os.path.dirname(lib)
    name = os.path.basename(lib)[3:-3]  # libX.so -> X
    subprocess.run([cc, '-std=c99', '-Wall', '-Werror', '-I', os.path.join(ROOT, 'include'), str(src),
                    '-L', libdir, '-l' + name, '-Wl,-rpath,' + libdir, '-o', str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    lines = r.stdout.splitlines()
    assert lines[1] == 'padded 272 272 channels 217 out 32 32 filters 43'
    groups = [l for l in lines if l.startswith('group ')]
    assert len(groups) == 7
    assert groups[0] == 'group 0 level 0 tasks 1 size 272x272 fold 1'
    assert 'size 136x136 fold 2' in groups[4]
