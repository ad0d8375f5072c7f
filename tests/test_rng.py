"""The counter-based generator of the GPU path tracers (csrc/rng.cuh) is
Philox-4x32-10: check it against the known-answer vectors published with
Random123 (Salmon et al., SC 2011), compiled for the host."""
import os
import shutil
import subprocess

import pytest

KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
    ((0xffffffff,) * 4, (0xffffffff, 0xffffffff), (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
    ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
     (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
]


def test_philox_known_answers(repo_dir, tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    src = tmp_path / "kat.cpp"
    lines = ["#define __host__", "#define __device__", "#define __forceinline__ inline",
             f'#include "{os.path.join(repo_dir, "lightmetrica-v2_gb300", "csrc", "rng.cuh")}"',
             "#include <cstdio>", "int main() {"]
    for c, k, _ in KAT:
        lines.append(f"  {{ auto r = lmgpu::philox4x32_10({c[0]}u, {c[1]}u, {c[2]}u, {c[3]}u, {k[0]}u, {k[1]}u);"
                     ' std::printf("%08x %08x %08x %08x\\n", r.v[0], r.v[1], r.v[2], r.v[3]); }')
    lines.append("  return 0; }")
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "kat"
    subprocess.run([cxx, "-O2", "-o", str(exe), str(src)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    for (_, _, expect), line in zip(KAT, out):
        assert line.split() == [f"{x:08x}" for x in expect]
