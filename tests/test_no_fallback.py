"""The product path has no CPU fallback and never routes through the oracle
(CPU only; skipped where a CUDA device is present).

Every public entry point that computes needs the CUDA library and a device:
without a device it raises GbmieError instead of computing on the host.  No
module of the package imports the oracle."""
import ast
import os

import numpy as np
import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.skipif(torch.cuda.is_available(), reason="checks the behaviour without a CUDA device")


def test_public_api_raises_without_a_device():
    from geosmie_gb300 import Mie, MultipleMie, gsf
    from geosmie_gb300._native import GbmieError
    from geosmie_gb300.table import TablePlan, run_tables
    from geosmie_gb300 import workloads
    with pytest.raises(GbmieError):
        Mie(m=complex(1.5, 0.01), x=2.5).qext()
    cost = np.cos(np.radians(np.linspace(0.0, 180.0, 7)))
    with pytest.raises(GbmieError):
        mm = MultipleMie(np.array([0.5, 1.0]), None, cost)
        mm.preCalculate()
        mm.calculateS12SizeRange(1.5, 0.01)
    spec, _ = workloads.homogeneous_single()
    with pytest.raises(GbmieError):
        TablePlan(spec)
    with pytest.raises(GbmieError):
        list(run_tables([spec]))
    with pytest.raises(GbmieError):
        gsf.expand(np.linspace(0.0, 180.0, 19), np.ones((1, 6, 19)))


def test_package_never_imports_the_oracle():
    pkg = os.path.join(ROOT, "geosmie_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if not f.endswith(".py"):
                continue
            tree = ast.parse(open(os.path.join(dirpath, f)).read())
            for node in ast.walk(tree):
                names = []
                if isinstance(node, ast.Import):
                    names = [a.name for a in node.names]
                elif isinstance(node, ast.ImportFrom):
                    names = [node.module or ""]
                assert not any(n == "oracle" or n.startswith("oracle.") for n in names), (f, names)


def test_bench_uses_the_oracle_only_in_its_cpu_legs():
    """bench.py reaches the oracle only from its CPU legs: the per-unit CPU
    task (_unit_task: the 1-core baseline and the accuracy check) and the
    reference arm (run_reference)."""
    tree = ast.parse(open(os.path.join(ROOT, "bench.py")).read())
    allowed = {"_unit_task", "run_reference"}
    seen = []

    def visit(node, fn):
        for child in ast.iter_child_nodes(node):
            name = child.name if isinstance(child, ast.FunctionDef) else fn
            mods = []
            if isinstance(child, ast.Import):
                mods = [a.name for a in child.names]
            elif isinstance(child, ast.ImportFrom):
                mods = [child.module or ""]
            if any(m == "oracle" or m.startswith("oracle.") for m in mods):
                seen.append(fn)
            visit(child, name)
    visit(tree, None)
    assert seen and set(seen) <= allowed, seen
