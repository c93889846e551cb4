"""Build and run helpers of the hostmpi oracle.  TEST INFRASTRUCTURE ONLY.

The oracle is a fork-per-rank host MPI (hostmpi/hostmpi.cpp) with the same
API subset as the device runtime and the reference's collective algorithms;
every workload program in dphpc-project_gb300/programs/ is compiled against
it (Makefile) and runs on the host cores as the checker of the GPU results.
Only the tests, the smoke check and the benchmark's CPU-baseline leg use this
module; the product library never links or runs anything here.
"""
from __future__ import annotations

import os
import subprocess
import sys
from dataclasses import dataclass

ORACLE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(ORACLE)
ORACLE_BIN = os.path.join(ORACLE, "build", "bin")


def _jobs() -> int:
    return max(1, min(32, os.cpu_count() or 1))


def build(verbose: bool = False, reference: bool = True) -> None:
    """Compile hostmpi and every workload program against it; with
    `reference`, also build the reference's own programs and their converted
    forms (ref.mk) when the reference tree is present."""
    out = None if verbose else subprocess.PIPE
    r = subprocess.run(["make", "-C", ORACLE, f"-j{_jobs()}"], stdout=out, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout or "")
        raise RuntimeError("oracle build failed")
    if reference:
        r = subprocess.run(["make", "-C", ORACLE, "-f", "ref.mk", "if-present"], stdout=out,
                           stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout or "")
            raise RuntimeError("reference programs against the oracle: build failed")


@dataclass
class RunResult:
    returncode: int
    stdout: str
    stderr: str

    def lines(self, prefix: str = "") -> list[str]:
        return [ln for ln in self.stdout.splitlines() if ln.startswith(prefix)]


def run_oracle(name: str, args: list[str] | None = None, nranks: int = 2,
               extra: list[str] | None = None, timeout: float = 300.0) -> RunResult:
    """Run a workload program on the host cores through hostmpi (one process per rank)."""
    exe = os.path.join(ORACLE_BIN, name)
    if not os.path.exists(exe):
        raise FileNotFoundError(f"{exe} is not built; run build() first")
    cmd = [exe, *(args or []), "---gpumpi", "-n", str(nranks), *(extra or [])]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=timeout)
    return RunResult(r.returncode, r.stdout, r.stderr)
