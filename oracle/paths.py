"""Where the test infrastructure finds FreeFEM: its source tree (to compile oracle/_ref and to
check that the plugin compiles against FreeFEM's headers) and a FreeFEM build (to generate the
golden fixtures and to run the plugin inside FreeFEM).  Every default is named here once and
each can be overridden by an environment variable.  Neither is needed on a GPU machine: the
GPU tests, the smoke test and the benchmark read the committed fixtures only."""
import os

# FreeFEM source tree (FreeFem-sources): FFGPU_REFERENCE
REFERENCE = os.environ.get("FFGPU_REFERENCE", "/root/reference")
# FreeFEM build tree with src/nw/FreeFem++-nw and plugin/seq/ff-c++: FREEFEM_BUILD
FREEFEM_BUILD = os.environ.get("FREEFEM_BUILD", "/tmp/ffbuild")
FF_BIN = os.environ.get("FREEFEM_BIN", os.path.join(FREEFEM_BUILD, "src", "nw", "FreeFem++-nw"))
FF_CXX = os.environ.get("FREEFEM_FFCXX", os.path.join(FREEFEM_BUILD, "plugin", "seq", "ff-c++"))
FF_LOADPATH = os.environ.get("FF_LOADPATH", os.path.join(FREEFEM_BUILD, "plugin", "seq"))
