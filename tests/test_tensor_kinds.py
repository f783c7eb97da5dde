"""Why the tensor kNN runs bf16 MMA: on sm_103a the integer MMA does not exist.

ptxas for sm_103a refuses tcgen05.mma .kind::i8 ("Feature '.kind::i8' not supported on
.target 'sm_103a'"), while it accepts .kind::f16 (the bf16 form the tensor engine issues)
and accepts .kind::i8 for sm_100a.  The u8/i8/4-bit codes are exact in bf16 and their dot
products over <= 128 codes are exact in the fp32 accumulator, so the bf16 form gives the
integer distances the reference computes.  Compiles a two-line kernel per case; no GPU."""
import os
import shutil
import subprocess

import pytest

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")

SRC = r'''
#include <cstdint>
__global__ void k(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                 " tcgen05.mma.cta_group::1.kind::KIND [%0], %1, %2, %3, p;\n}\n"
                 :: "r"(tmem), "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
'''


def _compile(tmp_path, kind, arch):
    src = tmp_path / f"mma_{kind}_{arch}.cu"
    src.write_text(SRC.replace("KIND", kind))
    r = subprocess.run([NVCC, "-gencode", f"arch=compute_{arch},code=sm_{arch}", "-c", str(src), "-o",
                        str(tmp_path / f"{kind}_{arch}.o")], capture_output=True, text=True, timeout=120)
    return r.returncode, r.stderr


@pytest.mark.skipif(not (os.path.exists(NVCC) or shutil.which("nvcc")), reason="nvcc not available")
def test_integer_mma_is_refused_on_sm_103a(tmp_path):
    rc, err = _compile(tmp_path, "i8", "103a")
    assert rc != 0 and "not supported" in err and "kind::i8" in err
    rc, err = _compile(tmp_path, "f16", "103a")
    assert rc == 0, err
    rc, err = _compile(tmp_path, "i8", "100a")
    assert rc == 0, err
