"""The C++ front end (include/randblas_gb300.hpp) as a RandBLAS caller would use it: a small C++
program is compiled against the header and the library and run on the host (no GPU needed for
the parts it exercises)."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_front_end(rb_host, tmp_path):
    lib_dir = os.path.join(ROOT, "randblas_gb300")
    exe = str(tmp_path / "cpp_api_check")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp_api_check.cc"), "-L", lib_dir,
                    "-lrandblas_gb300", "-Wl,-rpath," + lib_dir, "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.strip().endswith("ok"), out.stdout + out.stderr
