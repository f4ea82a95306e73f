"""The FP64-free rounding and square-root forms of the CUDA kernels against
the reference's double forms (tests/cpp/round_equiv.c): eflib's
fast_roundi / fast_floori / fast_ceili of a float argument and
vector_::length's double square root.  The CUDA kernels avoid FP64, which is
slow on this part; parity needs these to agree for every float.  This test
checks the boundary neighbourhoods, the small magnitudes densely and every
61st float; `round_equiv --all` checks all 2^32 (about two minutes)."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_float_forms_equal_double_forms(tmp_path):
    exe = str(tmp_path / "round_equiv")
    subprocess.run(["gcc", "-O2", "-frounding-math", "-o", exe, os.path.join(ROOT, "tests", "cpp", "round_equiv.c"),
                    "-lm"], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert " 0 differ" in r.stdout
