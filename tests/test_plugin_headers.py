"""The FreeFEM plugin (freefem-sources_gb300/plugin/ffgpu.cpp) compiles against FreeFEM's own
headers.  This runs wherever the FreeFEM sources are (oracle/paths.py) -- also where no FreeFEM
build exists to load the plugin into (test_plugin_freefem.py needs one).  config.h, written by
FreeFEM's configure step, is replaced by an empty stub, as oracle/Makefile does."""
import os
import shutil
import subprocess

import pytest

from paths import REFERENCE   # oracle/paths.py

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(REFERENCE, "src")

pytestmark = pytest.mark.skipif(not os.path.exists(os.path.join(SRC, "fflib", "ff++.hpp"))
                                or shutil.which("g++") is None, reason="FreeFEM sources not here")


def test_plugin_compiles_against_freefem_headers():
    stub = os.path.join(REPO, "oracle", "_build", "plugin_inc")
    os.makedirs(stub, exist_ok=True)
    open(os.path.join(stub, "config.h"), "w").close()
    inc = ["-I" + stub] + ["-I" + os.path.join(SRC, d) for d in ("fflib", "femlib", "Graphics", "Algo",
                                                               "lglib", "bamglib")]
    r = subprocess.run(["g++", "-std=c++14", "-fsyntax-only", "-Wall", *inc,
                        "-I" + os.path.join(REPO, "include"),
                        os.path.join(REPO, "freefem-sources_gb300", "plugin", "ffgpu.cpp")],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-4000:]
