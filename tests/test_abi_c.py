"""The C ABI from C, as a foreign-language binding uses it: a C99 program built
against include/basefold_gpu.h alone and linked to libbasefold_gpu.so takes
the address of every declared entry point and runs the verifier-only setup of
both schemes (device < 0: no GPU is touched), whose query counts and proof
sizes match the Python binding's."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


def declared_symbols():
    text = open(os.path.join(INCLUDE, "basefold_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bf_[a-z0-9_]+)\s*\(", text)))


def test_c_program_links_every_entry_point(built_lib, tmp_path):
    from basefold_gpu import BasefoldConfig, BinaryReedSolomonCode, _native, prime

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    names = declared_symbols()
    table = ",\n  ".join(f"(fn){n}" for n in names)
    src = tmp_path / "abi.c"
    src.write_text(f"""#include <stdio.h>
#include "basefold_gpu.h"
typedef void (*fn)(void);
static const fn entry[] = {{
  {table}
}};
int main(void) {{
  bf_pcs* p = NULL;
  bf_bb_pcs* q = NULL;
  if (bf_pcs_setup(-1, 128, 1, 10, NULL, &p) != BF_OK) return 1;
  if (bf_bb_pcs_setup(-1, 128, 1, 10, NULL, &q) != BF_OK) return 2;
  printf("%zu %zu %zu %zu %zu\\n", sizeof(entry) / sizeof(entry[0]), bf_pcs_num_queries(p),
         bf_pcs_proof_size(p, 1, 1), bf_bb_pcs_num_queries(q), bf_bb_pcs_proof_size(q, 3, 1));
  bf_pcs_free(p);
  bf_bb_pcs_free(q);
  return 0;
}}
""")
    libdir = os.path.dirname(_native.LIB_PATH)
    exe = tmp_path / "abi"
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Wpedantic", "-Werror", "-I", INCLUDE, str(src), "-o",
                    str(exe), "-L", libdir, "-lbasefold_gpu", f"-Wl,-rpath,{libdir}"], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    count, nq, size, bb_nq, bb_size = (int(v) for v in out)
    assert count == len(names)
    binary = built_lib.Basefold.setup(BasefoldConfig(BinaryReedSolomonCode(128, 1, 10)), device=-1)
    assert (nq, size) == (binary.num_queries(), binary.proof_size(1, 1))
    bb = prime.BabyBearBasefold.setup(BasefoldConfig(prime.ReedSolomonCode(128, 1, 10)), device=-1)
    assert (bb_nq, bb_size) == (bb.num_queries(), bb.proof_size(3, 1))
