"""A C program compiled against include/fsk.h and linked to libfsk.so, with
no Python in between, calls the host side of the ABI: the version, a status
string, a workspace size and the argument checks, which refuse null pointers
and a bad bandwidth with FSK_ERR_INVALID_ARGUMENT before any device work.
CPU only: none of these calls reaches the CUDA driver."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

C_SRC = r"""
#include <stdio.h>
#include <string.h>
#include "fsk.h"

int main(void) {
  if (fsk_version() <= 0) return 1;
  if (strstr(fsk_strerror(FSK_ERR_INVALID_ARGUMENT), "invalid") == NULL) return 2;
  const size_t ws = fsk_kde16_workspace_bytes(1024, 4096, 0);
  if (ws == 0) return 3;
  if (fsk_kde16(NULL, 1024, NULL, 4096, 1.0, 0, 1.0, 0.0, NULL, NULL, 0, NULL) != FSK_ERR_INVALID_ARGUMENT) return 4;
  const float dummy[16] = {0};
  float pdf[1], w[16];
  if (fsk_empscore16(dummy, 1, -1.0, FSK_SCORE_ORDERED, 0, pdf, w, NULL, 0, NULL) != FSK_ERR_INVALID_ARGUMENT)
    return 5;
  printf("ok %d %zu\n", fsk_version(), ws);
  return 0;
}
"""


def test_c_program_links_and_calls_the_abi(tmp_path):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    from fsk import _build

    lib = _build.build()
    src = tmp_path / "consumer.c"
    src.write_text(C_SRC)
    exe = tmp_path / "consumer"
    subprocess.run([gcc, "-std=c11", "-Wall", "-Werror", "-I", str(ROOT / "include"), str(src), "-o", str(exe),
                    "-L", str(lib.parent), "-lfsk", f"-Wl,-rpath,{lib.parent}"], check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert res.returncode == 0, (res.returncode, res.stdout, res.stderr)
    assert res.stdout.startswith("ok ")
