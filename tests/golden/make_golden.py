"""Generate the golden fixtures under tests/golden/ from the topomax reference.

Run where a topomax reference checkout is available, naming its root in
``TOPOMAX_REFERENCE`` (required; there is no default)::

    TOPOMAX_REFERENCE=/path/to/topomax python tests/golden/make_golden.py

It reads, without importing any reference module:

* ``designs/*.json`` (elasticity and fluid designs) -> ``tests/golden/designs/``;
* ``tests/test_data/FEM/triangle/data/correct_{data,rho}.dat`` -- the
  known answer of ``tests/test_elasticity_solver.py:30-55`` -- through an
  unpickler restricted to numpy types -> ``tests/golden/triangle_N10.json`` (the saved
  design vector kept in its file order: dolfin's serial CG1 dof order);
* ``tests/test_data/DEM/{short_cantilever,bridge}/problem_data.dat`` -- the
  known answers of ``tests/test_DEM_problem.py:14-43`` ->
  ``tests/golden/dem_<design>.npz``;
* ``designs/diffuser.json`` and ``tests/test_data/FEM/diffuser/data/correct_{data,rho}.dat``
  -- the known answer of ``tests/test_fluid_solver.py`` (the pickled ``IterationData``
  is read into a plain attribute holder) -> ``tests/golden/diffuser_N20.json``.

The fixtures are committed so the tests never need the reference at run time.
"""
from __future__ import annotations

import importlib
import json
import os
import pickle
import sys

import numpy as np

REF = os.environ.get("TOPOMAX_REFERENCE", "")
HERE = os.path.dirname(os.path.abspath(__file__))


class _NumpyOnly(pickle.Unpickler):
    def find_class(self, module, name):
        if module.split(".")[0] == "numpy":
            return getattr(importlib.import_module(module), name)
        raise pickle.UnpicklingError(f"refusing {module}.{name}")


def _load(path):
    with open(path, "rb") as f:
        return _NumpyOnly(f).load()


class _Record:
    """Holds the attributes of a pickled record (no methods, no reference code)."""

    def __setstate__(self, state):
        self.__dict__.update(state if isinstance(state, dict) else {"state": state})


class _RecordData(_NumpyOnly):
    def find_class(self, module, name):
        if (module, name) == ("src.utils", "IterationData"):
            return _Record
        return super().find_class(module, name)


def _load_record(path):
    with open(path, "rb") as f:
        return _RecordData(f).load()


def main():
    if not REF or not os.path.isdir(REF):
        sys.exit("set TOPOMAX_REFERENCE to the root of a topomax checkout"
                 + (f" ({REF} is not a directory)" if REF else ""))
    os.makedirs(os.path.join(HERE, "designs"), exist_ok=True)
    for name in sorted(os.listdir(os.path.join(REF, "designs"))):
        if not name.endswith(".json"):
            continue
        with open(os.path.join(REF, "designs", name)) as f:
            d = json.load(f)
        if "Elasticity" not in d and "Fluid" not in d:
            continue
        with open(os.path.join(HERE, "designs", name), "w") as f:
            json.dump(d, f, indent=2)

    base = os.path.join(REF, "tests", "test_data", "FEM", "triangle", "data")
    data = _load(os.path.join(base, "correct_data.dat"))
    rho = _load(os.path.join(base, "correct_rho.dat"))
    vec = np.asarray(rho["vector"], dtype=np.float64)
    out = {
        "design": "triangle.json",
        "N": int(rho["N"]),
        "objective": float(data["objective"]),
        "iteration": int(data["iteration"]),
        "penalty": float(data["penalty"]),
        "rho_sorted": np.sort(vec).tolist(),
        "rho_sum": float(vec.sum()),
        "rho_dolfin": vec.tolist(),
        "domain_size": [float(x) for x in rho["domain_size"]],
        "problem": str(rho["problem"]),
        "note": "rho_dolfin is the reference's saved design vector (dolfin's serial CG1 dof order)",
    }
    with open(os.path.join(HERE, "triangle_N10.json"), "w") as f:
        json.dump(out, f, indent=1)

    with open(os.path.join(REF, "designs", "diffuser.json")) as f:
        diffuser = json.load(f)
    with open(os.path.join(HERE, "designs", "diffuser.json"), "w") as f:
        json.dump(diffuser, f, indent=2)
    base = os.path.join(REF, "tests", "test_data", "FEM", "diffuser", "data")
    rec = _load_record(os.path.join(base, "correct_data.dat"))
    rho = _load(os.path.join(base, "correct_rho.dat"))
    vec = np.asarray(rho["vector"], dtype=np.float64)
    with open(os.path.join(HERE, "diffuser_N20.json"), "w") as f:
        json.dump({"design": "diffuser.json", "N": int(rho["N"]), "objective": float(rec.objective),
                   "iteration": int(rec.iteration), "penalty": float(rec.penalty),
                   "rho_sorted": np.sort(vec).tolist(), "rho_sum": float(vec.sum()),
                   "rho_dolfin": vec.tolist(), "domain_size": [float(x) for x in rho["domain_size"]],
                   "problem": str(rho["problem"]),
                   "note": "rho_dolfin is the reference's saved design vector (dolfin's serial CG1 dof order)"},
                  f, indent=1)

    for design in ("short_cantilever", "bridge"):
        p = os.path.join(REF, "tests", "test_data", "DEM", design, "problem_data.dat")
        if not os.path.exists(p):
            continue
        d = _load(p)
        np.savez(os.path.join(HERE, f"dem_{design}.npz"),
                 objective=np.float64(d["objective"]),
                 gradient=np.asarray(d["gradient"]))
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
