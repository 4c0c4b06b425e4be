"""The C++ drop-in classes (open-qmin_gb300/host/landauDeGennesLC_gb300.h and
energyMinimizerFIRE_gb300.h) compiled against the reference's own headers and
linked with the reference's CPU objects (built from its sources by the
oracle/ref recipe, with its single-rank mpi.h stand-in) and libqmin_gb300.so.

tests/dropin_reference_main.cpp sets up a lattice through the reference's
multirankSimulation exactly as its CLI does and runs two minimize() calls,
once with the reference's landauDeGennesLC + energyMinimizerFIRE and once
with the drop-in subclasses in their place.  With a CUDA device the two must
agree (FIRE iterations exact, forceMax and E/NActive to 1e-9); without one the
drop-in must reach the library through the reference's virtual calls and
report the missing device as an exception.  Skipped where the reference tree
is not present (it is not on GPU machines)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ITERS = 40


@pytest.fixture(scope="module")
def dropin_binary(qmin, tmp_path_factory):
    import __graft_entry__ as ge
    ref = ge.reference_tree()
    if not ref:
        pytest.skip("reference source tree not present")
    recipe = os.path.join(ROOT, "oracle", "ref")
    subprocess.run(["make", "-s", "-j8", "-C", recipe], check=True, stdout=subprocess.DEVNULL)
    lib = os.path.join(ROOT, "oracle", "_ref", "libqminref.a")
    assert os.path.exists(lib)
    out = str(tmp_path_factory.mktemp("dropin") / "dropin_reference_main")
    build_dir = os.path.join(ROOT, "open-qmin_gb300", "_build")
    incs = ["-I", recipe] + sum((["-I", os.path.join(ref, d)] for d in
                                 ["inc", "src/model", "src/forces", "src/simulation", "src/updaters",
                                  "src/utilities"]), [])
    cmd = (["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-DDIMENSION=5", "-w"] + incs
           + ["-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "open-qmin_gb300", "host"),
              os.path.join(ROOT, "tests", "dropin_reference_main.cpp"), lib, "-L", build_dir, "-lqmin_gb300",
              "-Wl,-rpath," + build_dir, "-o", out])
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return out


def _run(binary, mode):
    r = subprocess.run([binary, mode, str(ITERS)], capture_output=True, text=True, timeout=300)
    lines = [ln for ln in r.stdout.splitlines() if ln and (ln[0].isdigit() or ln.startswith("DROPIN_ERROR"))]
    return r.returncode, (lines[-1] if lines else r.stdout + r.stderr)


def _has_cuda():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_reference_path_runs(dropin_binary):
    rc, line = _run(dropin_binary, "ref")
    assert rc == 0, line
    it, fm, e = line.split()
    assert int(it) == ITERS and float(fm) > 0 and abs(float(e)) < 1e3


def test_dropin_matches_reference_or_reports_missing_device(dropin_binary):
    rc, line = _run(dropin_binary, "gb300")
    if not _has_cuda():
        assert rc == 3 and line.startswith("DROPIN_ERROR"), line
        assert "qmin_create" in line and "no CUDA device" in line, line
        return
    assert rc == 0, line
    rc0, ref = _run(dropin_binary, "ref")
    it, fm, e = (float(x) for x in line.split())
    it0, fm0, e0 = (float(x) for x in ref.split())
    assert it == it0
    assert abs(fm - fm0) <= 1e-9 * fm0
    assert abs(e - e0) <= 1e-9 * abs(e0)
