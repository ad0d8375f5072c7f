"""The C-ABI library builds, loads and exports every entry point declared in
include/*.h.  No compute call is made: on a machine without a GPU the only
call exercised must fail loudly with LMGPU_ERR_NO_DEVICE (no CPU fallback)."""
import ctypes
import glob
import os
import re
import subprocess

import pytest


def declared_symbols(repo_dir):
    syms = set()
    for h in glob.glob(os.path.join(repo_dir, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(lmgpu_\w+)\s*\(", src, flags=re.M):
            syms.add(m.group(1))
    return syms


def test_header_declares_entry_points(repo_dir):
    syms = declared_symbols(repo_dir)
    for s in ("lmgpu_accel_create", "lmgpu_accel_build", "lmgpu_trace", "lmgpu_trace_device"):
        assert s in syms


def test_library_exports_all_declared_symbols(gpu_lib, repo_dir):
    from lmgpu.build import LIB_PATH

    out = subprocess.run(["nm", "-D", "--defined-only", LIB_PATH], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = declared_symbols(repo_dir) - exported
    assert not missing, f"declared but not exported: {sorted(missing)}"
    L = ctypes.CDLL(LIB_PATH)
    for s in declared_symbols(repo_dir):
        assert hasattr(L, s)


def test_version_string(gpu_lib):
    assert "sm_103a" in gpu_lib.version()


def test_no_cpu_fallback_without_gpu(gpu_lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is visible; covered by the gpu tests")
    with pytest.raises(gpu_lib.LmgpuError) as e:
        gpu_lib.Accel()
    assert e.value.code == 5


def test_null_arguments_rejected(gpu_lib):
    L = gpu_lib.lib()
    assert L.lmgpu_accel_create(None) == 1
    assert L.lmgpu_trace(None, None, None, 0, 0) == 1
    assert L.lmgpu_accel_get_info(None, None) == 1
    assert L.lmgpu_scene_set_trace_profile(None, 1) == 1
    assert L.lmgpu_scene_read_trace_profile(None, None) == 1
    assert L.lmgpu_batch_set_trace_profile(None, 1) == 1
    assert L.lmgpu_batch_read_trace_profile(None, None) == 1
    assert L.lmgpu_last_error()


@pytest.mark.parametrize("plugin", ["accel_cuda", "renderer_pt_cuda", "renderer_ptmis_cuda", "renderer_ptdirect_cuda",
                                    "renderer_ltdirect_cuda", "renderer_bdpt_cuda", "renderer_pt_guided_cuda",
                                    "renderer_vcm_cuda"])
def test_reference_plugin_compiles_against_reference_headers(repo_dir, reference_root, plugin):
    """plugin/*.cpp, the bindings a maintainer adds to the reference tree
    (accel::cuda, renderer::pt_cuda, renderer::ptmis_cuda,
    renderer::ptdirect_cuda, renderer::ltdirect_cuda, renderer::bdpt_cuda,
    renderer::pt_guided_cuda),
    compile against the
    reference's own headers (x86-64 only: the reference forces SSE)."""
    import platform
    import shutil

    ref = os.path.join(reference_root, "include")
    if not os.path.isdir(ref) or platform.machine() != "x86_64" or not shutil.which("g++"):
        pytest.skip("reference headers or x86-64 g++ not available")
    src = os.path.join(repo_dir, "lightmetrica-v2_gb300", "plugin", plugin + ".cpp")
    cmd = ["g++", "-std=c++14", "-fsyntax-only", "-w", "-DLM_USE_SINGLE_PRECISION", "-msse4.2",
           "-I", os.path.join(repo_dir, "oracle", "refharness", "shim"), "-I", ref,
           "-I", os.path.join(repo_dir, "include"), src]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
