"""The reference drivers' file formats (disorder files, result .dat files)."""
import shutil
import subprocess

import numpy as np
import pytest


def cxx_format(tmp_path, values):
    """How a C++ ostream with precision(10) prints the values (the reference
    drivers' outfile.precision(10)), one per line."""
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "fmt.cpp"
    src.write_text('#include <iostream>\n#include <cstdlib>\nint main(int c, char** v) {\n'
                   '  std::cout.precision(10);\n'
                   '  for (int i = 1; i < c; ++i) std::cout << std::strtod(v[i], nullptr) << "\\n";\n}\n')
    exe = tmp_path / "fmt"
    subprocess.run([cxx, "-O1", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)] + [repr(float(v)) for v in values], capture_output=True, text=True, check=True)
    return out.stdout.splitlines()


def test_number_format_matches_cxx_ostream(tmp_path, edlib):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import datio
    vals = [-29.62437941471926, 0.1234567891234, 1e-5, -3.25e-12, 123456789012.5, 0.0, 1.0, -0.5, 7.0 / 3.0,
            2.0 ** 70, -1.0e-300]
    assert [datio.fmt10(v) for v in vals] == cxx_format(tmp_path, vals)


def test_random_numbers_file_round_trip(tmp_path, edlib):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import datio
    a = datio.random_numbers(3, 18, seed=7)
    assert a.shape == (3, 18) and np.all(np.abs(a) < 1.0)
    fn = datio.write_random_numbers(str(tmp_path), "Lieb", a)
    assert fn.endswith("randNum_Lieb-L18.dat")
    datio.write_random_numbers(str(tmp_path), "Lieb", a[:1])  # append, no second header
    lines = open(fn).read().splitlines()
    assert lines[0] == datio.RANDNUM_HEADER and len(lines) == 5
    assert sum(l.startswith("#") for l in lines) == 1
    assert lines[1].endswith("\t") and lines[1].count("\t") == 18
    b = datio.read_random_numbers(str(tmp_path), "Lieb", 18)
    assert b.shape == (4, 18)
    assert np.max(np.abs(b[:3] - a)) < 1e-9 and np.array_equal(b[3], b[0])
    r = datio.site_factors(b[0], 0.5)
    assert np.allclose(r, 1.0 + 0.5 * b[0])


def test_result_file_append_mode(tmp_path):
    from exact_diagonalization_for_fermionic_systems_with_gpu_gb300 import datio
    fn = datio.drude_filename(str(tmp_path), 12, "8", "6", "0.5")
    assert fn.endswith("DrudeWeight_v2_Kagome-L12aU8Q6X0.5.dat")
    datio.append_rows(fn, datio.DRUDE_HEADER, [(-29.62437941471926, 0.25, 0.125, 0.1875)])
    datio.append_rows(fn, datio.DRUDE_HEADER, [(-1.0, 2.0, 3.0, 2.5)])
    lines = open(fn).read().splitlines()
    assert lines == [datio.DRUDE_HEADER, "\t-29.62437941\t0.25\t0.125\t0.1875", "\t-1\t2\t3\t2.5"]
