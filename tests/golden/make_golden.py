"""Regenerate tests/golden/cpi_pi.txt from the reference's own pi program.

The reference ships MPICH's example toolchain_tests/pi/cpi.c as its pi test.
This script compiles that file by path, unmodified, against the hostmpi
oracle (a host MPI with rank-order reductions) and records the program's
result line for several interval counts and rank counts.  The fixture pins
the oracle and the GPU runtime to the reference program's output.

Usage: python tests/golden/make_golden.py [REFERENCE_ROOT]
(default: the tree oracle/ref.mk names, GPUMPI_REFERENCE_TREE overriding it)
"""
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CASES = [(1000, 1), (100000, 3), (100000, 8), (10000000, 8), (1000003, 64)]


def build_cpi(ref_root: str, out_dir: str) -> str:
    src = os.path.join(ref_root, "toolchain_tests", "pi", "cpi.c")
    oracle = os.path.join(ROOT, "oracle")
    subprocess.run(["make", "-C", oracle, "build/libhostmpi.a"], check=True, capture_output=True)
    exe = os.path.join(out_dir, "cpi")
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-I", os.path.join(oracle, "hostmpi", "include"),
                    "-Dmain=hostmpi_user_main", src, os.path.join(oracle, "build", "libhostmpi.a"),
                    "-lstdc++", "-lpthread", "-lm", "-o", exe], check=True)
    return exe


def run_cases(exe: str) -> list[str]:
    lines = []
    for n, ranks in CASES:
        out = subprocess.run([exe, str(n), "---gpumpi", "-n", str(ranks)], capture_output=True, text=True,
                             timeout=600, check=True).stdout
        pi = [ln for ln in out.splitlines() if ln.startswith("pi is approximately")]
        lines.append(f"{n} {ranks} | {pi[0]}")
    return lines


def main() -> None:
    if len(sys.argv) > 1:
        ref_root = sys.argv[1]
    else:
        ref_root = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "-f", "ref.mk", "print-ref"],
                                  capture_output=True, text=True, check=True).stdout.strip()
    with tempfile.TemporaryDirectory() as d:
        lines = run_cases(build_cpi(ref_root, d))
    with open(os.path.join(HERE, "cpi_pi.txt"), "w") as f:
        f.write("# n ranks | result line of the reference's toolchain_tests/pi/cpi.c on the hostmpi oracle\n")
        f.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
