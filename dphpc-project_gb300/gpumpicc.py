#!/usr/bin/env python3
"""Compiler wrapper for MPI C programs on the device MPI runtime, in place of
scripts/gpumpicc.py (used as `MPICC` of an existing build).

    gpumpicc.py [--max-ranks N] [--malloc-version V] [--project DIR] [--outdir DIR]
                sources... [compiler options] [-- compiler options]
    MPICC=".../gpumpicc.py" make ...

Each C source (.c/.cpp/.cxx) is converted by `gpumpi_convert` (foo.c -> foo.cu;
project headers h -> h.cuh), beside the source unless --outdir is given, then
compiled by nvcc for sm_103a; a `.cu` file is taken as already converted.  Without -c the runtime (launcher entry, host
`main`, runtime library) is linked in; with no sources the call only links.
Compiler options are filtered as gpumpicc.py:40-67 does: -I and -D are kept,
-c and -o honoured, object files passed on; everything else (optimisation
flags, -lm, ...) is dropped.  The project directory (the headers to convert)
is GPU_MPI_PROJECT, as for the clang tool, else the source's directory.
"""

from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "build")
sys.path.insert(0, HERE)

import gpumpi_convert as conv  # noqa: E402

SOURCE_EXT = (".c", ".cpp", ".cxx")
NVCC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
# The runtime library is built with a 64-register cap; programs linked into its
# kernel must not exceed it.  -fmad=false keeps FP64 results equal to a host build.
NVFLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O3", "-rdc=true",
           "-fmad=false", "-maxrregcount=64", "-diag-suppress=177,2464,550"]
RUNTIME = [os.path.join(BUILD, "prog_entry.o"), os.path.join(BUILD, "prog_main.o"),
           "-L" + BUILD, "-lgpumpi_rt"]


def split_args(args):
    """(sources, converter options, compiler options)."""
    sources, copts, cc = [], {}, []
    it = iter(args)
    for a in it:
        if a == "--":
            continue
        if a in ("--max-ranks", "--malloc-version", "--malloc_version", "--project", "--outdir"):
            copts[a.lstrip("-").replace("_", "-")] = next(it)
        elif a.split("=", 1)[0] in ("--max-ranks", "--malloc-version", "--malloc_version", "--project", "--outdir"):
            k, v = a.split("=", 1)
            copts[k.lstrip("-").replace("_", "-")] = v
        elif a.lower().endswith(SOURCE_EXT + (".cu",)) and not a.startswith("-"):
            sources.append(a)
        else:
            cc.append(a)
    return sources, copts, cc


def filter_compile_args(cc):
    """Keep -I/-D (joined or separate), -c, -o X and object files."""
    out, incdirs = [], []
    it = iter(cc)
    for a in it:
        if a in ("-I", "-D"):
            v = next(it)
            out.append(a + v)
            if a == "-I":
                incdirs.append(v)
        elif a.startswith(("-I", "-D")):
            out.append(a)
            if a.startswith("-I"):
                incdirs.append(a[2:])
        elif a == "-c":
            out.append(a)
        elif a == "-o":
            out += [a, next(it)]
        elif a.endswith((".o", ".a")):
            out.append(a)
    return out, incdirs


def main(argv=None) -> int:
    argv = sys.argv[1:] if argv is None else argv
    sources, copts, cc = split_args(argv)
    args, incdirs = filter_compile_args(cc)
    opts = conv.Options(
        max_ranks=int(copts.get("max-ranks", os.environ.get("GPU_MPI_MAX_RANKS", conv.DEFAULT_MAX_RANKS))),
        malloc_version=int(copts.get("malloc-version", 0)))
    outdir = copts.get("outdir")
    cu_files = []
    for src in sources:
        if src.endswith(".cu"):
            cu_files.append(src)
            continue
        project = os.path.realpath(copts.get("project") or os.environ.get("GPU_MPI_PROJECT")
                                   or os.path.dirname(os.path.abspath(src)))
        try:
            res = conv.convert_tu(src, opts, project, incdirs)
        except conv.ConvertError as e:
            print("gpumpicc: %s" % e, file=sys.stderr)
            return 1
        for path, text in res.items():
            dst = conv.output_name(path, src)
            if outdir and dst.startswith(project + os.sep):
                dst = os.path.join(outdir, os.path.relpath(dst, project))
                os.makedirs(os.path.dirname(dst), exist_ok=True)
            with open(dst, "w") as f:
                f.write(text)
            if path == os.path.realpath(src):
                cu_files.append(dst)
    link = "-c" not in args
    if link:
        missing = [p for p in RUNTIME[:2] + [os.path.join(BUILD, "libgpumpi_rt.a")] if not os.path.exists(p)]
        if missing:
            print("gpumpicc: runtime not built (%s); run make -C %s" % (", ".join(missing), HERE), file=sys.stderr)
            return 1
    if "-c" in args and len(cu_files) == 1 and "-o" not in args:
        # nvcc names the object after the .cu file; keep the name the build expects (foo.c -> foo.o)
        args += ["-o", os.path.splitext(os.path.basename(sources[0]))[0] + ".o"]
    cmd = [NVCC] + NVFLAGS + cu_files + args + ["-I" + os.path.join(ROOT, "include", "gpumpi"),
                                                "-I" + os.path.join(ROOT, "include")]
    if link:
        cmd += RUNTIME
    return subprocess.run(cmd).returncode


if __name__ == "__main__":
    sys.exit(main())
