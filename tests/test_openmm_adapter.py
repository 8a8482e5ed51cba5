"""The OpenMM plugin adapter (openmm_plugin/) compiled and run on the CPU.

OpenMM is not installed here, so the adapter is compiled against stand-in
OpenMM headers (tests/openmm_stub/include: the members of OpenMM's core,
CUDA platform and the plugin's force and kernel classes that it touches) and
linked with a recording stand-in of the gbx C ABI.  The driver then walks
OpenMM's plugin protocol -- registerKernelFactories(), createKernelImpl(),
initialize / execute / copyParametersToContext -- and checks the calls the
adapter makes: the atom order handed over before the first step and after
each reorder (parameters are not re-sent), the flags of each OpenMM
precision mode, the box and global-parameter updates, an earlier step's
overflowed table surfacing as an OpenMMException, a force outside the
canonical expression set handed to gbx_create_custom with its global
parameters followed, a force's exclusions, term types and energy parameter
derivatives passed on (the derivatives summed into the context's workspace
each step), Continuous1DFunction tables passed on and other tabulated
function types refused, and the refusal of CustomIntegral.
"""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STUB = os.path.join(REPO, "tests", "openmm_stub")
PLUGIN = os.path.join(REPO, "openmmcustomgbintegralforce_gb300", "openmm_plugin")
CUDA_INC = os.environ.get("CUDA_HOME", "/usr/local/cuda") + "/include"


def test_adapter_follows_the_plugin_protocol(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None or not os.path.exists(os.path.join(CUDA_INC, "cuda.h")):
        pytest.skip("needs g++ and the CUDA headers")
    exe = str(tmp_path / "adapter_driver")
    cmd = [gxx, "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(STUB, "include"), "-I",
           os.path.join(REPO, "include"), "-I", PLUGIN, "-I", CUDA_INC,
           os.path.join(PLUGIN, "GB300CharmmKernels.cpp"), os.path.join(PLUGIN, "GB300CharmmKernelFactory.cpp"),
           os.path.join(STUB, "fake_gbx.cpp"), os.path.join(STUB, "adapter_driver.cpp"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL OK" in r.stdout
