"""Compiles the C++ RelBuilder driver (tests/cpp/relbuilder_main.cpp)
against the in-tree library into a temporary directory."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_driver(tmpdir) -> str:
    lib_dir = os.path.join(ROOT, "proteus_gb300")
    cuda = "/usr/local/cuda"
    out = os.path.join(str(tmpdir), "relbuilder_main")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"),
                    "-I" + os.path.join(cuda, "include"), os.path.join(ROOT, "tests", "cpp", "relbuilder_main.cpp"),
                    "-o", out, "-L" + lib_dir, "-l:libgbjoin.so", "-Wl,-rpath," + lib_dir,
                    "-L" + os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath," + os.path.join(cuda, "lib64")],
                   check=True)
    return out
