"""Source converter (dphpc-project_gb300/gpumpi_convert.py), on the CPU.

Rules: each rewrite of source_converter/converter.cpp checked on a small
input.  Semantics: the converter's test programs (tests/convert_cases/*.c)
run unmodified and converted on the hostmpi oracle and print the same lines;
their converted forms compile for sm_103a.  Reference programs (when the
reference tree is present): cpi.c, global_var.c, NPB IS and NPB DT pass
through the converter and still give the reference's answers on the oracle.
"""
import os
import subprocess

import pytest

from conftest import _load, reference_tree

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = os.path.join(ROOT, "tests", "convert_cases")
ORACLE = os.path.join(ROOT, "oracle")
REF = reference_tree()
NVCC = "/usr/local/cuda/bin/nvcc"
CASE_OPTS = {"globals": 0, "ring": 0, "coalesce": 3, "fileio": 0}


@pytest.fixture(scope="module")
def conv():
    return _load("gpumpi_convert", "dphpc-project_gb300/gpumpi_convert.py")


def C(conv, src, **kw):
    return conv.convert_source(src, conv.Options(max_ranks=kw.pop("ranks", 4), **kw))


def squash(s):
    return " ".join(s.split())


# ---------------------------------------------------------------- rules


def test_main_and_functions_become_device_code(conv):
    out = C(conv, "int f(int);\nint f(int a) { return a; }\nint main(int ac, char *av[]) { return f(ac); }\n")
    assert out.startswith('#include "global_vars.cuh"\n')
    assert "__device__ int f(int);" in out
    assert "__device__ int f(int a)" in out
    # main keeps its parameter names, so the body still reads them
    assert "__device__ int __gpu_main(int ac, char** av)" in out
    assert "__device__ int __gpu_max_threads() {\n    return 4;\n}" in out
    out = C(conv, "int main(void) { return 0; }")
    assert "__gpu_main(int argc, char** argv)" in out


def test_globals_are_replicated_and_wrapped(conv):
    out = C(conv, "int g = -15;\nint a[2] = {1, 2};\nint *p;\nint f(void) { g++; return a[1] + *p; }\n")
    assert "__device__ int g[4] = {-15, -15, -15, -15};" in out
    assert "__device__ int a[4][2] = {{1, 2}, {1, 2}, {1, 2}, {1, 2}};" in out
    assert "__device__ int *p[4];" in out
    assert "__gpu_global(g)++;" in out
    assert "return __gpu_global(a)[1] + *__gpu_global(p);" in out


def test_extern_unsized_string_and_address_initialisers(conv):
    out = C(conv, 'extern int g;\nint g = 1;\nint v[] = {1, 2, 3};\nchar s[] = "ab";\nint *q = &g;\n')
    assert "__device__ extern int g[4];" in out
    assert "int v[4][3] = {{1, 2, 3}," in out  # the size the clang tool leaves out
    assert 'char s[4][sizeof("ab")] = {"ab", "ab", "ab", "ab"};' in out
    # each rank's pointer points at its own copy
    assert "int *q[4] = {&g[0], &g[1], &g[2], &g[3]};" in out


def test_read_only_globals_are_not_replicated(conv):
    out = C(conv, "const int lim[2] = {1, 2};\nconst char *names[2] = {\"a\", \"b\"};\n"
                  "int f(void) { return lim[0] + names[1][0]; }")
    assert "__device__ const int lim[2] = {1, 2};" in out
    # an array of pointers to const is itself writable: replicated
    assert "const char *names[4][2]" in out
    assert "return lim[0] + __gpu_global(names)[1][0];" in out


def test_function_statics_and_shadowing(conv):
    src = """int x = 1;
int f(int x) { return x; }
int g(void) {
    static int calls = 0;
    int r = x;
    { int x = 5; r += x; }
    for (int x = 0; x < 2; x++) r += x;
    calls++;
    return r + x + calls;
}
"""
    out = C(conv, src)
    assert "int f(int x) { return x; }" in out
    assert "__device__ static int calls[4] = {0, 0, 0, 0};" in out
    assert "int r = __gpu_global(x);" in out
    assert "{ int x = 5; r += x; }" in out
    assert "for (int x = 0; x < 2; x++) r += x;" in out
    assert "__gpu_global(calls)++;" in out
    assert "return r + __gpu_global(x) + __gpu_global(calls);" in out


def test_macros_members_and_labels(conv):
    src = """#define G2 g2
#define ADD(g2, y) ((g2) + (y))
struct s { int g2; };
int g2;
int f(struct s *p) {
    G2 = p->g2;
    goto g2;
g2:
    return ADD(1, g2);
}
"""
    out = C(conv, src)
    assert "#define G2 __gpu_global(g2)" in out
    assert "#define ADD(g2, y) ((g2) + (y))" in out  # a macro parameter, not the global
    assert "G2 = p->g2;" in out
    assert "goto g2;" in out and "\ng2:" in out
    assert "return ADD(1, __gpu_global(g2));" in out


def test_old_style_definitions(conv):
    out = C(conv, "int add(a, b)\n    int a;\n    double *b;\n{\n    return a + (int)*b;\n}\n")
    assert "__device__ int add(int a, double *b)" in squash(out)
    assert "int a;" not in out


def test_void_pointer_conversions_get_casts(conv):
    src = """#include <stdlib.h>
struct node { struct node *next; double *vals; };
double *mk(int n) { return malloc(n * sizeof(double)); }
void use(int *p);
int *g;
void f(void) {
    struct node *n = malloc(sizeof *n);
    void *raw = malloc(8);
    int **rows = calloc(2, sizeof(int *));
    n->vals = malloc(8);
    g = raw;
    rows[0] = malloc(4);
    use(malloc(4));
    free(raw);
}
"""
    out = C(conv, src)
    assert "return (double *)malloc(n * sizeof(double));" in out
    assert "struct node *n = (struct node *)malloc(sizeof *n);" in out
    assert "void *raw = malloc(8);" in out
    assert "int **rows = (int **)calloc(2, sizeof(int *));" in out
    assert "n->vals = (double *)malloc(8);" in out
    assert "__gpu_global(g) = (int *)raw;" in out
    assert "rows[0] = (int *)malloc(4);" in out
    assert "use((int *)malloc(4));" in out
    # a `void *` struct member read into a typed pointer, and returned as one
    out = C(conv, "typedef struct { void *head; } Q;\nint *first(Q *q) { int *h;\n h = q->head;\n return q->head; }\n")
    assert "h = (int *)q->head;" in out
    assert "return (int *)q->head;" in out


def test_cxx_keywords_restrict_includes_and_dead_code(conv):
    src = """#include <stdio.h>
#include "local.h"
#if 0
int class_unused = undefined_thing(;
#endif
int class = 2;
void cp(double * restrict a, const double * restrict b) { a[0] = b[0]; }
int f(int new) { return class + new; }
"""
    out = C(conv, src)
    assert "#include <stdio.h.cuh>" in out and '#include "local.h.cuh"' in out
    assert "int class_unused = undefined_thing(;" in out  # left as written
    assert "__device__ int __decl_class[4]" in out
    assert "double * __restrict__ a" in out
    assert "int f(int __decl_new) { return __gpu_global(__decl_class) + __decl_new; }" in out


def test_empty_prototype_takes_the_definition_parameters(conv):
    out = C(conv, "double h();\ndouble h(double x, int n) { return x * n; }\n")
    assert "__device__ double h(double x, int n);" in out


def test_allocator_version_rewrites(conv):
    src = """#include <stdlib.h>
#include <mpi.h>
int *mk(void);
int *mk(void) { return malloc(4); }
int *cond(int n) { if (n) return malloc(4); return 0; }
void ex(int *s, int *r) { MPI_Alltoall(s, 1, MPI_INT, r, 1, MPI_INT, MPI_COMM_WORLD); }
int use(void) { int *p = mk(); free(p); return 0; }
int main(int argc, char **argv) {
    int *p = malloc(8);
    ex(p, p + 1);
    if (argc > 1) { free(mk()); }
    use();
    return 0;
}
"""
    out = C(conv, src, malloc_version=3)
    assert out.startswith('#define GPUMPI_MALLOC_V3\n#include "global_vars.cuh"\n')
    assert "int *mk(bool __coalesced = false);" in out
    assert "int *mk(bool __coalesced) { return (int *)malloc(4, __coalesced); }" in out
    assert "int *cond(int n) { if (n) return (int *)malloc(4); return 0; }" in out
    assert "void ex(int *s, int *r, bool __coalesced = false)" in out
    assert "MPI_Alltoall_coalesce(s, 1, MPI_INT, r, 1, MPI_INT, MPI_COMM_WORLD, __coalesced);" in out
    assert "int *p = mk(false);" in out  # `use` has no flag of its own
    assert "int *p = (int *)malloc(8, true);" in out
    assert "ex(p, p + 1, true);" in out
    assert "free(mk());" in out  # conditional: unchanged
    assert "__gpu_init_malloc();" in out
    assert "__gpu_clean_malloc();\n    return 0;" in out


def test_unsupported_forms_are_reported(conv):
    with pytest.raises(conv.ConvertError):
        C(conv, "int a[] = {[2] = 1};\n")
    with pytest.raises(conv.ConvertError):
        C(conv, "int f(void) { return (1; }\n")


# ---------------------------------------------------------------- semantics on the oracle


def _run(exe, n, timeout=120, cwd=None):
    r = subprocess.run([exe, "---gpumpi", "-n", str(n)], capture_output=True, text=True, timeout=timeout,
                       cwd=cwd)
    assert r.returncode == 0, r.stderr[-2000:]
    return r.stdout


@pytest.fixture(scope="module")
def case_builds(oracle_built, tmp_path_factory):
    d = tmp_path_factory.mktemp("convert_cases")
    lib = os.path.join(ORACLE, "build", "libhostmpi.a")
    inc = os.path.join(ORACLE, "hostmpi", "include")
    out = {}
    for name, mv in CASE_OPTS.items():
        src = os.path.join(CASES, name + ".c")
        orig = str(d / (name + "_orig"))
        r = subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-Dmain=hostmpi_user_main", "-I" + inc, src, lib,
                            "-lstdc++", "-lpthread", "-lm", "-o", orig], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        r = subprocess.run(["python3", os.path.join(ROOT, "dphpc-project_gb300", "gpumpi_convert.py"), src,
                            "--max-ranks", "64", "--malloc-version", str(mv), "--outdir", str(d),
                            "--project", CASES], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        cu = str(d / (name + ".cu"))
        conv_exe = str(d / (name + "_conv"))
        r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-x", "c++", "-I" + inc, cu, "-x",
                            "none", lib, "-lpthread", "-o", conv_exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        out[name] = (orig, conv_exe, cu)
    return out


@pytest.mark.parametrize("name", sorted(CASE_OPTS))
@pytest.mark.parametrize("ranks", [1, 3, 8])
def test_converted_cases_match_the_original_on_the_oracle(case_builds, name, ranks, tmp_path):
    orig, conv_exe, _ = case_builds[name]
    (tmp_path / "a").mkdir()
    (tmp_path / "b").mkdir()
    a = _run(orig, ranks, cwd=str(tmp_path / "a"))   # fileio.c writes in its working directory
    assert a.strip()
    assert _run(conv_exe, ranks, cwd=str(tmp_path / "b")) == a


@pytest.mark.skipif(not os.path.exists(NVCC), reason="nvcc absent")
@pytest.mark.parametrize("name", sorted(CASE_OPTS))
def test_converted_cases_compile_for_sm103a(case_builds, name, tmp_path):
    cu = case_builds[name][2]
    r = subprocess.run([NVCC, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O3", "-rdc=true",
                        "-fmad=false", "-maxrregcount=64", "-I" + os.path.join(ROOT, "include", "gpumpi"),
                        "-I" + os.path.join(ROOT, "include"), "-c", cu, "-o", str(tmp_path / "x.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


# ---------------------------------------------------------------- the reference's programs

NPBDEFS = ['-DNPBVERSION="3.4.1"', '-DCOMPILETIME="n/a"', '-DMPICC="gcc"', '-DCFLAGS="-O2"', '-DCLINK="gcc"',
           '-DCLINKFLAGS=""', '-DCMPI_LIB="hostmpi"', '-DCMPI_INC=""']


def _unstable(line):
    return "Time in seconds" in line or "Mop/s" in line


@pytest.fixture(scope="module")
def ref_conv(oracle_built):
    if REF is None:
        pytest.skip("reference tree absent")
    r = subprocess.run(["make", "-C", ORACLE, "-f", "ref.mk", f"REF={REF}", "all", "conv"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    return os.path.join(ORACLE, "_ref")


def _host_build(srcs, exe, extra=()):
    inc = os.path.join(ORACLE, "hostmpi", "include")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-w", "-x", "c++", "-I" + inc, *extra,
                        *srcs, "-x", "none", os.path.join(ORACLE, "build", "libhostmpi.a"), "-lpthread", "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def test_converted_reference_cpi_prints_the_golden_lines(ref_conv, tmp_path):
    exe = _host_build([os.path.join(ref_conv, "conv", "cpi", "cpi.cu")], str(tmp_path / "cpi"))
    for line in open(os.path.join(ROOT, "tests", "golden", "cpi_pi.txt")):
        if line.startswith("#") or not line.strip():
            continue
        key, expect = line.rstrip("\n").split(" | ")
        n, ranks = key.split()
        r = subprocess.run([exe, n, "---gpumpi", "-n", ranks], capture_output=True, text=True, timeout=120)
        assert r.returncode == 0
        assert expect in r.stdout


def test_converted_reference_global_var_passes(ref_conv, tmp_path):
    exe = _host_build([os.path.join(ref_conv, "conv", "global_var", "global_var.cu")], str(tmp_path / "gv"))
    r = subprocess.run([exe, "---gpumpi", "-n", "4"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "error" not in r.stdout


@pytest.mark.parametrize("graph,ranks", [("BH", 5), ("WH", 8), ("SH", 12)])
def test_converted_reference_npb_dt_matches_the_unmodified_build(ref_conv, tmp_path, graph, ranks):
    npb = os.path.join(ref_conv, "conv", "npb")
    exe = _host_build([os.path.join(npb, "DT", "dt.cu"), os.path.join(npb, "DT", "DGraph.cu"),
                       os.path.join(npb, "common", "randdp.cu"), os.path.join(npb, "common", "c_print_results.cu"),
                       os.path.join(npb, "common", "c_timers.cu")], str(tmp_path / "dt"),
                      ["-I" + os.path.join(ref_conv, "conv", "dt_S")] + NPBDEFS)
    run = lambda e: subprocess.run([e, graph, "---gpumpi", "-n", str(ranks)], capture_output=True, text=True,
                                   timeout=300)  # noqa: E731
    got, want = run(exe), run(os.path.join(ref_conv, "dt.S"))
    assert got.returncode == 0 and want.returncode == 0
    assert "Verification    =               SUCCESSFUL" in got.stdout
    strip = lambda s: [x for x in s.splitlines() if not _unstable(x)]  # noqa: E731
    assert strip(got.stdout) == strip(want.stdout)


@pytest.mark.parametrize("cls,ranks", [("S", 2), ("W", 4)])
def test_converted_reference_npb_is_matches_the_unmodified_build(ref_conv, tmp_path, cls, ranks):
    npb = os.path.join(ref_conv, "conv", "npb")
    exe = _host_build([os.path.join(npb, "IS", "is.cu"), os.path.join(npb, "common", "c_print_results.cu"),
                       os.path.join(npb, "common", "c_timers.cu")], str(tmp_path / "is"),
                      ["-I" + os.path.join(ref_conv, "conv", "is_" + cls)] + NPBDEFS)
    got = _run(exe, ranks, timeout=300)
    want = _run(os.path.join(ref_conv, "is." + cls), ranks, timeout=300)
    assert "Verification    =               SUCCESSFUL" in got
    strip = lambda s: [x for x in s.splitlines() if not _unstable(x)]  # noqa: E731
    assert strip(got) == strip(want)
