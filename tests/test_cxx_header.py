"""include/pbrinkman.hpp: a caller written against the reference's interface
(its matrix types from the stand-in matrix.h, readData with its driver's
defaults, periodicBrinkman / fftBrinkman with their reference signatures)
compiles unchanged and runs through the C ABI; the parameter-file readers
(readData's map form, cuda/periodicBrinkman.cu:44-70, and array twin,
cuda/periodicBrinkman.h:524-554) read the reference's format."""
import os
import shutil
import subprocess

import pytest

from periodicbrinkman_gb300 import _lib
from periodicbrinkman_gb300.api import read_data, read_data_array

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PARAMS = "Lx: 1.0\nLy:   1.0\n\nLz: 1\nd: 0.125\ne: 0.01\nalpha: 10\nM: 2\nunknown 3.5\nalpha: 12\n"


def _build(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    exe = str(tmp_path / "reference_caller")
    libdir = os.path.dirname(_lib.lib_path())
    subprocess.run([gxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I",
                    os.path.join(ROOT, "oracle", "ref_shim", "include"), "-I", os.path.join(cuda, "include"),
                    os.path.join(ROOT, "tests", "cxx", "reference_caller.cpp"), "-o", exe, "-L", libdir,
                    "-lpbrinkman", "-Wl,-rpath," + libdir, "-L", os.path.join(cuda, "lib64"), "-lcudart"],
                   check=True)
    p = tmp_path / "param.txt"
    p.write_text(PARAMS)
    return exe, str(p)


def _run(exe, *args):
    out = subprocess.run([exe, *args], capture_output=True, text=True, check=True).stdout
    return out.splitlines()


def test_reference_style_caller_compiles_and_reads_params(tmp_path):
    exe, param = _build(tmp_path)
    lines = _run(exe, param)
    got = {tuple(l.split()[:2]): float(l.split()[2]) for l in lines if l.startswith(("map ", "array "))}
    # file values override the driver's defaults; a later line overrides an earlier one
    assert got[("map", "alpha")] == 12.0 and got[("map", "d")] == 0.125 and got[("map", "M")] == 2.0
    assert got[("map", "boxSize")] == 1.0 and got[("map", "unknown")] == 3.5
    assert got[("array", "e")] == 0.01 and got[("array", "toPrint")] == 0.0
    assert "missing 1" in lines
    if _lib.device_count() == 0:  # no GPU: the C ABI's error comes back as a pbrinkman::error
        assert any(l.startswith(f"error {_lib.PB_ERR_CUDA}") for l in lines), lines


def test_param_readers_python(tmp_path):
    p = tmp_path / "param.txt"
    p.write_text(PARAMS)
    d = read_data(p, {"Lx": 9.0, "boxSize": 1.0})
    assert d == {"Lx": 1.0, "Ly": 1.0, "Lz": 1.0, "d": 0.125, "e": 0.01, "alpha": 12.0, "M": 2.0, "unknown": 3.5,
                 "boxSize": 1.0}
    v = read_data_array(p, ["alpha", "nothere", "d"], [0.0, 7.0, 0.0])
    assert list(v) == [12.0, 7.0, 0.125]
    q = tmp_path / "comma.txt"
    q.write_text("a,1.5\n,b,,2\n")  # strtok: runs of delimiters separate, leading ones are skipped
    assert read_data(q, delimiters=",") == {"a": 1.5, "b": 2.0}
    bad = tmp_path / "bad.txt"
    bad.write_text("alpha:\n")
    with pytest.raises(_lib.PbError):
        read_data(bad)
    with pytest.raises(_lib.PbError):
        read_data(tmp_path / "absent.txt")


@pytest.mark.gpu
def test_reference_style_caller_on_gpu(tmp_path):
    exe, param = _build(tmp_path)
    lines = _run(exe, param, "gpu")
    fft = [l for l in lines if l.startswith("fftBrinkman diff")]
    dense = [l for l in lines if l.startswith("periodicBrinkman diff")]
    assert fft and float(fft[0].split()[2]) == 0.0, lines
    assert dense and float(dense[0].split()[2]) <= 1e-13 * float(dense[0].split()[4]), lines
    assert f"shape error {_lib.PB_ERR_INVALID}" in lines
