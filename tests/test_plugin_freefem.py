"""The FreeFEM plugin compiled with FreeFEM's own ff-c++ and loaded into FreeFEM.

Needs a FreeFEM installation (FREEFEM_BIN, FREEFEM_FFCXX; defaults are the from-source build
used for the golden fixtures) and is skipped without one.  Without a GPU the device solver
must stop the script with FreeFEM's ExecError -- never fall back to a CPU solve."""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FF_BIN = os.environ.get("FREEFEM_BIN", "/tmp/ffbuild/src/nw/FreeFem++-nw")
FF_CXX = os.environ.get("FREEFEM_FFCXX", "/tmp/ffbuild/plugin/seq/ff-c++")
FF_LOADPATH = os.environ.get("FF_LOADPATH", "/tmp/ffbuild/plugin/seq")

pytestmark = pytest.mark.skipif(not (os.path.exists(FF_BIN) and os.path.exists(FF_CXX)),
                                reason="FreeFEM is not installed here")

SCRIPT = r"""
load "%s"
mesh Th=square(8,8);
fespace Vh(Th,P1);
Vh u,v;
varf a(u,v)=int2d(Th,qft=qf2pT)(dx(u)*dx(v)+dy(u)*dy(v)) + int2d(Th,qft=qf2pT)(1.*v) + on(1,2,3,4,u=0);
matrix A=a(Vh,Vh,solver=GPUCG,eps=1e-10);
real[int] b=a(0,Vh);
u[]=0; u[]=A^-1*b;
cout << "umax " << u[].max << endl;
"""


def test_plugin_registers_solvers_and_refuses_cpu_fallback(tmp_path):
    from ffgpu.build import build
    lib = build()
    src = tmp_path / "ffgpu.cpp"
    shutil.copy(os.path.join(REPO, "freefem-sources_gb300", "plugin", "ffgpu.cpp"), src)
    r = subprocess.run([FF_CXX, "-auto", "ffgpu.cpp", "-I" + os.path.join(REPO, "include"), lib],
                       cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and (tmp_path / "ffgpu.so").exists(), r.stdout + r.stderr
    (tmp_path / "t.edp").write_text(SCRIPT % str(tmp_path / "ffgpu"))
    env = dict(os.environ, FF_LOADPATH=FF_LOADPATH,
               LD_LIBRARY_PATH=os.path.dirname(lib) + ":" + os.environ.get("LD_LIBRARY_PATH", ""))
    r = subprocess.run([FF_BIN, "-nw", "t.edp", "-v", "2"], cwd=tmp_path, env=env, capture_output=True,
                       text=True, timeout=300)
    out = r.stdout + r.stderr
    assert "load: ffgpu (GPUCG, GPUGMRES, GPUCGMIXED)" in out
    import torch
    if torch.cuda.is_available():
        assert r.returncode == 0 and "umax 0.07" in out, out[-2000:]
    else:
        assert r.returncode != 0
        assert "ffgpu: no usable CUDA device" in out
        # (-v 2 echoes the script, so look for the printed value, not the word)
        assert not any(line.startswith("umax ") for line in r.stdout.splitlines())
