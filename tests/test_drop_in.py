"""The C++ drop-in: callers written against the reference's public headers
build unchanged against include/ and libnasoq_gb300.so.

  * (CPU) the reference's own examples (examples/lbl_main.cpp,
    lbl_somod_main.cpp, nasoq_main.cpp) compile and link unchanged, when the
    reference sources are present (NASOQ_REFERENCE, default /root/reference);
  * (CPU) every method the reference declares on SolverSettings
    (include/nasoq/QP/linear_solver_wrapper.h) and Nasoq (include/nasoq/nasoq.h)
    is declared by the drop-in headers too;
  * (GPU) tests/callers/solver_settings_flow.cpp, a caller of both
    SolverSettings modes and of the maintenance methods, runs and its printed
    solutions match dense solves of the same systems."""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

import nasoq_gb300 as nq

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("NASOQ_REFERENCE", "/root/reference")
CALLER = os.path.join(ROOT, "tests", "callers", "solver_settings_flow.cpp")
LIBDIR = os.path.dirname(nq.LIB_PATH)


def _cuda_lib():
    for d in ("/usr/local/cuda/lib64", "/usr/local/cuda/targets/sbsa-linux/lib",
              "/usr/local/cuda/targets/x86_64-linux/lib"):
        if os.path.isdir(d):
            return d
    return None


def build_program(src, out):
    """g++ src against include/ and the library; returns (rc, stderr)."""
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), src, "-o", out, "-L", LIBDIR,
           "-lnasoq_gb300", f"-Wl,-rpath,{LIBDIR}"]
    cl = _cuda_lib()
    if cl:
        cmd.append(f"-Wl,-rpath-link,{cl}")
    p = subprocess.run(cmd, capture_output=True, text=True)
    return p.returncode, p.stderr


needs_gxx = pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
needs_ref = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "examples")),
                               reason="reference sources not present")


@needs_gxx
@needs_ref
@pytest.mark.parametrize("example", ["lbl_main", "lbl_somod_main", "nasoq_main"])
def test_reference_examples_build_unchanged(example, tmp_path):
    rc, err = build_program(os.path.join(REF, "examples", example + ".cpp"), str(tmp_path / example))
    assert rc == 0, err[-2000:]


def _methods(header, struct):
    """Names of the methods a struct declares (or defines inline); the
    CHOLMOD-only block (#ifdef CHOLROWMOD) is not part of the default build."""
    txt = open(header).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    txt = re.sub(r"//[^\n]*", "", txt)
    txt = re.sub(r"#ifdef\s+CHOLROWMOD.*?#endif", "", txt, flags=re.S)
    m = re.search(r"struct\s+" + struct + r"\s*\{", txt)
    assert m, f"{struct} not found in {header}"
    depth, j, body = 1, m.end(), []
    while depth and j < len(txt):  # the struct body with inline function bodies blanked
        ch = txt[j]
        if ch == "{":
            depth += 1
            if depth == 2:
                body.append(";")
        elif ch == "}":
            depth -= 1
        elif depth == 1:
            body.append(ch)
        j += 1
    names = set(re.findall(r"\b([A-Za-z_]\w*)\s*\([^;{}]*\)\s*(?:const\s*)?;", "".join(body)))
    return {n for n in names if n not in (struct, "~" + struct)}


@needs_ref
@pytest.mark.parametrize("header,struct", [("include/nasoq/QP/linear_solver_wrapper.h", "SolverSettings"),
                                           ("include/nasoq/nasoq.h", "Nasoq")])
def test_drop_in_declares_every_reference_method(header, struct):
    ref = _methods(os.path.join(REF, header), struct)
    ours = _methods(os.path.join(ROOT, header), struct)
    assert len(ref) > 10
    missing = sorted(ref - ours)
    assert not missing, f"{struct}: methods missing from the drop-in: {missing}"


@needs_gxx
def test_caller_links(tmp_path):
    rc, err = build_program(CALLER, str(tmp_path / "flow"))
    assert rc == 0, err[-2000:]


def _parse(out):
    res = {}
    for line in out.splitlines():
        if ":" not in line:
            continue
        k, v = line.split(":", 1)
        res[k.strip()] = [float(t) for t in v.split()]
    return res


def _kkt_solution(H, q, B, d, active):
    n, m = H.shape[0], B.shape[0]
    S = [k for k in range(m) if k in active]
    Kd = np.zeros((n + len(S), n + len(S)))
    Kd[:n, :n] = H
    Kd[n:, :n] = B[S]
    Kd[:n, n:] = B[S].T
    sol = np.linalg.solve(Kd, np.concatenate([q, d[S]]))
    full = np.zeros(n + m)
    full[:n] = sol[:n]
    for t, k in enumerate(S):
        full[n + k] = sol[n + t]
    return full


@needs_gxx
@pytest.mark.gpu
def test_caller_runs_both_modes(tmp_path):
    exe = str(tmp_path / "flow")
    rc, err = build_program(CALLER, exe)
    assert rc == 0, err[-2000:]
    p = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stdout + p.stderr
    r = _parse(p.stdout)
    K = np.array([[4, 1, 0, 1], [1, 3, 1, 0], [0, 1, -2, 1], [1, 0, 1, -3]], float)
    b1, b2 = np.array([1, 2, 3, 4.0]), np.array([-1, 0.5, 2, 0.0])
    assert np.allclose(r["x1"], np.linalg.solve(K, b1), rtol=0, atol=1e-12)
    assert np.allclose(r["x2"], np.linalg.solve(K, b2), rtol=0, atol=1e-12)
    assert r["bwd_err"][0] <= 1e-15
    # refinement alone from x0 = b2 reaches the same solution (two restarts x two steps on 4 unknowns)
    assert np.allclose(r["xr"], np.linalg.solve(K, b2), rtol=0, atol=1e-10)
    assert r["check"] == [1.0]
    assert sorted(int(v) for v in r["perm"]) == [0, 1, 2, 3]
    # lower triangle of the factor, diagonal included, in simplicial form
    assert r["simplicial_nnz"][0] >= 4
    levels, last, nsuper = (int(v) for v in r["levels"])
    assert levels >= 1 and last == nsuper
    assert all(v > 0 for v in r["workspace"])
    assert r["stubs"] == [1.0] * 5
    H = np.array([[3, 1], [1, 2.0]])
    q = np.array([-1, -2.0])
    B = np.array([[1, 0], [1, 1.0]])
    d = np.array([0.5, 1.0])
    for key, act in (("m1_none", ()), ("m1_row0", (0,)), ("m1_rows01", (0, 1)), ("m1_row1", (1,))):
        assert np.allclose(r[key], _kkt_solution(H, q, B, d, act), rtol=0, atol=1e-9), key
