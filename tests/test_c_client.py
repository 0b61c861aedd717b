"""The C ABI from a C program: include/nqueens_gb300.h compiles as strict C99 (and as C++), and a client
linked against libnqgpu.so runs the host-only entry points with the results the Python binding gives.
No GPU call is made (the generator, the start list and the status strings run on the host)."""
import os
import shutil
import subprocess

import pytest

from conftest import REPO

CLIENT = r"""
#include <stdio.h>
#include <stdlib.h>
#include "nqueens_gb300.h"

int main(void) {
  const int N = 14;
  int64_t ns = nq_start_constellations(N, NULL, 0);
  int32_t *starts = (int32_t *)malloc(sizeof(int32_t) * (size_t)ns);
  if (nq_start_constellations(N, starts, ns) != ns) return 2;
  int64_t m = nq_gen_constellations(N, nq_preset_for(N), NULL, 0);
  nq_record *rec = (nq_record *)malloc(sizeof(nq_record) * (size_t)m);
  if (nq_gen_constellations(N, nq_preset_for(N), rec, m) != m) return 3;
  /* the records of the first 100 starts are the list's first records */
  int64_t k = nq_gen_constellations_starts(N, 0, 0, 100, NULL, 0);
  nq_record *part = (nq_record *)malloc(sizeof(nq_record) * (size_t)k);
  if (nq_gen_constellations_starts(N, 0, 0, 100, part, k) != k) return 4;
  for (int64_t i = 0; i < k; i++)
    if (part[i].ld != rec[i].ld || part[i].rd != rec[i].rd || part[i].col != rec[i].col ||
        part[i].startijkl != rec[i].startijkl) return 5;
  unsigned long long x = 0;
  for (int64_t i = 0; i < m; i++) x = x * 1000003ull + rec[i].ld + 3ull * rec[i].rd + 7ull * rec[i].col + rec[i].startijkl;
  printf("%s|%d|%lld|%d|%lld|%lld|%llu|%s|%s\n", nq_version(), nq_preset_for(N), (long long)ns, starts[0],
         (long long)m, (long long)k, x, nq_strerror(NQ_EPRESET), nq_strerror(NQ_OK));
  printf("%lld %lld\n", (long long)nq_start_constellations(5, NULL, 0),
         (long long)nq_gen_constellations_starts(N, 0, ns, 1, NULL, 0));
  free(starts); free(rec); free(part);
  return 0;
}
"""


def _lib_dir():
    from nqueens import _lib
    _lib.lib()
    return os.path.dirname(os.path.abspath(_lib.LIB_PATH))


@pytest.mark.parametrize("compiler,std", [("gcc", "-std=c99"), ("g++", "-std=c++17")])
def test_c_client_uses_the_header_and_library(tmp_path, compiler, std):
    if shutil.which(compiler) is None:
        pytest.skip(f"{compiler} not found")
    import nqueens
    libdir = _lib_dir()
    src = tmp_path / ("client.c" if compiler == "gcc" else "client.cpp")
    src.write_text(CLIENT)
    exe = tmp_path / "client"
    subprocess.run([compiler, std, "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", os.path.join(REPO, "include"),
                    str(src), "-o", str(exe), "-L", libdir, "-lnqgpu", f"-Wl,-rpath,{libdir}"], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines()
    f = out[0].split("|")
    N = 14
    recs = nqueens.gen_records(N)
    x = 0
    for r in recs.tolist():
        x = (x * 1000003 + r[0] + 3 * r[1] + 7 * r[2] + r[3]) % (1 << 64)
    starts = nqueens.start_constellations(N)
    assert f[0] == nqueens.lib().nq_version().decode()
    assert int(f[1]) == nqueens.select_dynamic_preset_queens(N)
    assert int(f[2]) == len(starts) and int(f[3]) == int(starts[0])
    assert int(f[4]) == len(recs)
    assert int(f[5]) == len(nqueens.gen_records_starts(N, 0, 100))
    assert int(f[6]) == x
    assert f[7] == "preset too deep for N" and f[8] == "ok"
    assert out[1] == "-1 -1"                     # N=5 has no start list here; a range past the end is NQ_EINVAL
