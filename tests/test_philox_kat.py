"""The shared Philox4x32-10 (include/rh_philox.h), built for the host, against
the known-answer vectors published with the Random123 library of Salmon,
Moraes, Dror and Shaw (SC'11), which defined the generator.  The GPU side is
pinned against cuRAND's Philox in tests/test_gpu_philox.py."""
import os
import subprocess
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# (counter c0..c3, key k0 k1) -> output words
KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF), (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


def test_host_philox_matches_published_vectors():
    calls = "".join(
        "{rh_u32x4 r=rh_philox4x32_10(%uu,%uu,%uu,%uu,%uu,%uu);"
        'printf("%%08x %%08x %%08x %%08x\\n",r.w[0],r.w[1],r.w[2],r.w[3]);}' % (c + k)
        for c, k, _ in KAT)
    src = '#include "rh_philox.h"\n#include <stdio.h>\nint main(void){%s return 0;}\n' % calls
    with tempfile.TemporaryDirectory() as d:
        c_file, exe = os.path.join(d, "kat.c"), os.path.join(d, "kat")
        open(c_file, "w").write(src)
        subprocess.run(["gcc", "-O2", "-I", os.path.join(ROOT, "include"), c_file, "-o", exe],
                       check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    got = [int(x, 16) for x in out]
    want = [w for _, _, ws in KAT for w in ws]
    assert got == want


def test_stream_blocks_are_philox_of_the_stream_counter():
    """rh_stream draws: block d>>1 of counter (d>>1, pos, step_lo, step_hi) and
    key (seed, cell); draw d uses half d&1 of it (the layout the oracle and
    the kernels share)."""
    src = r'''
#include "rh_philox.h"
#include <stdio.h>
int main(void) {
  rh_stream s; rh_stream_init(&s, 7u, 3u, 12345u, 0x100000002ull);
  int bad = 0;
  for (uint32_t d = 0; d < 8; ++d) {
    uint32_t hi, lo; rh_stream_next(&s, &hi, &lo);
    rh_u32x4 b = rh_philox4x32_10(d >> 1, 12345u, 2u, 1u, 7u, 3u);
    if (lo != b.w[2 * (d & 1)] || hi != b.w[2 * (d & 1) + 1]) bad++;
  }
  printf("%d\n", bad);
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c_file, exe = os.path.join(d, "s.c"), os.path.join(d, "s")
        open(c_file, "w").write(src)
        subprocess.run(["gcc", "-O2", "-I", os.path.join(ROOT, "include"), c_file, "-o", exe],
                       check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.strip()
    assert out == "0"
