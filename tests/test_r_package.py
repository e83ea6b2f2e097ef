"""R packaging of the engine, checked without R (R is absent on these machines).

accrqa_gb300/rpkg assembles an R source package from the reference's R code
(unchanged) and this engine's sources, with a configure script and a
Makevars template that build AccRQA.so for sm_103a.  Here:
  * the package assembles, and configure writes src/Makevars with the sm_103a
    nvcc rule, every source as an object and the static CUDA runtime;
  * the R registration (R_init_AccRQA in bindings.cpp, built with
    -DACCRQA_R_FOUND) compiles against stand-in declarations of the few R API
    names it uses and exports R_init_AccRQA;
  * every .C routine the reference's R code calls (R/RAccRQA.R) is registered
    with the number of arguments that call passes.
Skips where the reference tree is absent.
"""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

R_STUB = """
#ifndef R_STUB_H
#define R_STUB_H
typedef void *(*DL_FUNC)(void);
typedef struct { const char *name; DL_FUNC fun; int numArgs; void *types; } R_CMethodDef;
typedef struct _DllInfo DllInfo;
#ifdef __cplusplus
extern "C" {
#endif
int R_registerRoutines(DllInfo *, const R_CMethodDef *, const void *, const void *,
                       const void *);
int R_useDynamicSymbols(DllInfo *, int);
#ifdef __cplusplus
}
#endif
#define FALSE 0
#endif
"""


def _reference():
    tree = os.environ.get("ACCRQA_REFERENCE_TREE")
    if not tree:
        import __graft_entry__
        tree = __graft_entry__._REFERENCE_TREE
    return tree if os.path.isfile(os.path.join(tree, "R", "RAccRQA.R")) else None


@pytest.fixture(scope="module")
def pkg(tmp_path_factory):
    ref = _reference()
    if ref is None:
        pytest.skip("the reference's source tree is not present")
    from accrqa_gb300.rpkg import assemble
    out = str(tmp_path_factory.mktemp("rpkg") / "AccRQA")
    assemble.assemble(ref, out)
    return ref, out


def test_configure_writes_the_sm103a_makevars(pkg):
    from accrqa_gb300 import build
    _, out = pkg
    for f in ("DESCRIPTION", "NAMESPACE", "R/RAccRQA.R", "configure", "src/Makevars.in",
              "src/bindings.cpp", "src/accrqa_gb300.h"):
        assert os.path.exists(os.path.join(out, f)), f
    env = dict(os.environ, CUDA_HOME=build.cuda_home())
    r = subprocess.run(["sh", "configure"], cwd=out, env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    mk = open(os.path.join(out, "src", "Makevars")).read()
    assert "-gencode arch=compute_103a,code=sm_103a" in mk
    assert "-lcudart_static" in mk and "-DACCRQA_R_FOUND" in mk
    objs = set(re.search(r"^OBJECTS = (.*)$", mk, re.M).group(1).split())
    srcs = {os.path.splitext(f)[0] + ".o" for f in os.listdir(os.path.join(out, "src"))
            if f.endswith((".cpp", ".cu"))}
    assert objs == srcs


def test_configure_refuses_a_build_without_nvcc(pkg, tmp_path):
    _, out = pkg
    env = {"PATH": "/usr/bin:/bin", "CUDA_HOME": str(tmp_path / "none")}
    if any(os.path.exists(os.path.join(d, "nvcc")) for d in ("/usr/bin", "/bin")):
        pytest.skip("nvcc is on the minimal PATH")
    r = subprocess.run(["sh", "configure"], cwd=out, env=env, capture_output=True, text=True)
    assert r.returncode != 0 and "nvcc not found" in r.stderr


def test_registration_compiles_and_matches_the_r_calls(pkg, tmp_path):
    from accrqa_gb300 import build
    ref, out = pkg
    stub = tmp_path / "rstub"
    (stub / "R_ext").mkdir(parents=True)
    (stub / "R.h").write_text(R_STUB)
    (stub / "R_ext" / "Rdynload.h").write_text(R_STUB)
    obj = tmp_path / "bindings.o"
    r = subprocess.run(["g++", "-std=c++17", "-c", "-DACCRQA_R_FOUND", "-I", str(stub),
                        "-I", os.path.join(out, "src"),
                        "-I", os.path.join(build.cuda_home(), "include"),
                        os.path.join(out, "src", "bindings.cpp"), "-o", str(obj)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    syms = subprocess.run(["nm", "-g", "--defined-only", str(obj)], capture_output=True,
                          text=True).stdout
    assert re.search(r"\bR_init_AccRQA\b", syms)

    src = open(os.path.join(out, "src", "bindings.cpp")).read()
    registered = {m.group(1): int(m.group(2)) for m in
                  re.finditer(r'\{"(\w+)",\s*\(DL_FUNC\)&\w+,\s*(\d+)\}', src)}
    rcode = open(os.path.join(ref, "R", "RAccRQA.R")).read()
    calls = 0
    for m in re.finditer(r'\.C\("(\w+)",(.*?)\n\s*\)', rcode, re.S):
        name, body = m.group(1), m.group(2)
        nargs = len(re.findall(r"^\s*\w+\s*=", body, re.M))
        assert registered.get(name) == nargs, (name, nargs, registered.get(name))
        calls += 1
    assert calls >= 4
