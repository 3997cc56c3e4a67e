"""The C++ drop-in header compiles against the C ABI header alone (no GPU)."""
import subprocess

from conftest import ROOT


def test_algorithm_gpu_header_compiles(tmp_path):
    src = tmp_path / "t.cpp"
    src.write_text('#include "mlbm/Algorithm_gpu.h"\n'
                   'int main() { mlbm_config c; mlbm_config_init(&c); return c.lattice; }\n')
    subprocess.run(["g++", "-std=c++17", "-fsyntax-only", f"-I{ROOT / 'include'}", str(src)],
                   check=True)


def test_routine_driver_compiles(tmp_path):
    subprocess.run(["g++", "-std=c++17", "-fsyntax-only", f"-I{ROOT / 'include'}",
                    str(ROOT / "metalbm_gb300" / "cpp" / "routine_gpu.cpp")], check=True)
