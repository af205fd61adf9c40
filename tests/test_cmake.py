"""LibreTT's CMake surface: the package builds and installs with CMake and a
consumer links it the way it links LibreTT (LibreTT src/CMakeLists.txt:65-94,
cmake/librett-config.cmake.in): find_package(librett), target
librett::librett, headers under include/librett.  CPU only (nvcc
cross-compiles for sm_103a; nothing runs on a device)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

CONSUMER_CMAKE = """cmake_minimum_required(VERSION 3.22)
project(consumer LANGUAGES CXX)
find_package(librett REQUIRED)
add_executable(app app.cpp)
target_link_libraries(app PRIVATE librett::librett)
"""

CONSUMER_APP = """#include <librett/librett.h>
#include "librett_c.h"
int main() {
  librettHandle h;
  int dim[3] = {64, 48, 32}, perm[3] = {2, 0, 1};
  cudaStream_t s = 0;
  librettInitialize();
  librettResult r = librettPlan(&h, 3, dim, perm, sizeof(float), s);
  if (r == LIBRETT_SUCCESS) librettDestroy(h);
  librettFinalize();
  return librett_c_launch_count() == 0 ? 0 : 1;
}
"""


def _run(cmd, cwd):
    res = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True, timeout=900)
    assert res.returncode == 0, (cmd, res.stdout[-3000:], res.stderr[-3000:])


def test_cmake_package_and_consumer(tmp_path):
    if shutil.which("cmake") is None or shutil.which("nvcc") is None:
        pytest.skip("cmake or nvcc not available")
    gen = ["-G", "Ninja"] if shutil.which("ninja") else []
    prefix = tmp_path / "prefix"
    _run(["cmake", "-S", str(ROOT), "-B", str(tmp_path / "build"), *gen,
          f"-DCMAKE_INSTALL_PREFIX={prefix}"], tmp_path)
    _run(["cmake", "--build", str(tmp_path / "build"), "-j", "8"], tmp_path)
    _run(["cmake", "--install", str(tmp_path / "build")], tmp_path)
    lib = next(prefix.glob("lib*/librett.so"))
    assert (lib.parent / "models" / "plan_mlp.bin").exists()
    assert (prefix / "include" / "librett" / "librett.h").exists()
    nm = subprocess.run(["nm", "-D", "--defined-only", str(lib)], capture_output=True,
                        text=True, check=True).stdout
    assert "_Z11librettPlanPjiPiS0_mRP11CUstream_st" in nm
    app = tmp_path / "consumer"
    app.mkdir()
    (app / "CMakeLists.txt").write_text(CONSUMER_CMAKE)
    (app / "app.cpp").write_text(CONSUMER_APP)
    _run(["cmake", "-S", str(app), "-B", str(app / "build"), *gen,
          f"-DCMAKE_PREFIX_PATH={prefix}"], app)
    _run(["cmake", "--build", str(app / "build")], app)
    assert (app / "build" / "app").exists()
