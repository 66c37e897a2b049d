"""The shared Philox4x32-10 provider (include/rh_philox.h) against cuRAND's
own Philox4x32-10 generator, run on the GPU; and the host build of the same
header against the device build."""
import os
import subprocess
import tempfile

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_philox_matches_curand():
    src = os.path.join(ROOT, "tests", "cuda", "philox_curand.cu")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "philox_curand")
        subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-I",
                        os.path.join(ROOT, "include"), src, "-o", exe], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    lines = out.strip().splitlines()
    assert len(lines) == 10
    for ln in lines:
        f = ln.split()
        assert f[4:8] == f[9:13], ln


def test_host_and_device_philox_agree():
    import ctypes as C
    from oracle import oracle as O  # the oracle uses the host build of the header
    assert O.lib() is not None
    src = os.path.join(ROOT, "tests", "cuda", "philox_curand.cu")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "p")
        subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-I",
                        os.path.join(ROOT, "include"), src, "-o", exe], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    # host build: the same header compiled by gcc through a tiny C program
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "h.c")
        open(c, "w").write('#include "rh_philox.h"\n#include <stdio.h>\n'
                           'int main(){unsigned long long s[][2]={{0,0},{18,0},{18,977},'
                           '{1,123456789},{0xdeadbeefcafef00dull,5}};'
                           'for(int q=0;q<5;q++)for(int i=0;i<2;i++){rh_u32x4 a='
                           'rh_philox4x32_10(i,0,(uint32_t)s[q][1],(uint32_t)(s[q][1]>>32),'
                           '(uint32_t)s[q][0],(uint32_t)(s[q][0]>>32));'
                           'printf("%08x %08x %08x %08x\\n",a.w[0],a.w[1],a.w[2],a.w[3]);}}\n')
        exe = os.path.join(d, "h")
        subprocess.run(["gcc", "-O2", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        host = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split("\n")
    dev = [" ".join(ln.split()[9:13]) for ln in out.strip().splitlines()]
    assert dev == [h for h in host if h]
