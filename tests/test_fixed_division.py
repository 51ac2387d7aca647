"""The division sequence the neighbour passes use for the fixed divisors h and h^2,
checked on the host: verification on one binade covers every dividend in
[2^-100, 2^100] (the range the passes use it on without a range test), and the sign of
a zero quotient is restored (CPU)."""
import subprocess

from conftest import REPO

SRC = REPO / "tests" / "cpp" / "fixed_div_check.c"


def test_one_binade_verification_covers_the_unguarded_range(tmp_path):
    exe = tmp_path / "fixed_div_check"
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", str(SRC), "-o", str(exe), "-lm"],
                   check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    ok, nver, tested = out.stdout.split()
    assert ok == "ok" and int(nver) >= 4 and int(tested) >= 4 * (1 << 19)
