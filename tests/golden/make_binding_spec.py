"""Extract the reference's ctypes binding of its CUDA library into a fixture.

The reference drives its exports from Python through ctypes, in
CuSuperHelium/Python/integration/rhs.py (SimulationManager, rhs.py:68-340).
That module cannot be imported on Linux (it raises on a non-Windows os.name and
imports Windows-only ctypes pieces, matplotlib and h5py), so this script reads
it as text: it parses the file with `ast` and records, for every
`self.lib.<symbol>.argtypes = ...` and `.restype = ...`, the argument types
exactly as written, plus the field lists of the ctypes Structures the
signatures pass (CSimulationProperties, CGaussLegendreProperties, CRK4Options,
COptomechanicalProperties).  The tests rebuild the binding from this fixture
and drive libsfd.so through it.

Usage: SFD_REFERENCE_DIR=<reference checkout> python tests/golden/make_binding_spec.py [--check]
  writes tests/golden/ref_rhs_bindings.json (--check: compare instead of writing)
"""
import argparse
import ast
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REL = os.path.join("CuSuperHelium", "Python", "integration", "rhs.py")
OUT = os.path.join(HERE, "ref_rhs_bindings.json")


def _type(node):
    """A JSON descriptor of one ctypes type expression of rhs.py."""
    if isinstance(node, ast.Name):
        return {"kind": "name", "name": node.id}
    if isinstance(node, ast.Attribute):  # np.complex128
        return {"kind": "name", "name": node.attr}
    if isinstance(node, ast.Call) and isinstance(node.func, ast.Name):
        f = node.func.id
        if f == "POINTER":
            return {"kind": "pointer", "to": _type(node.args[0])}
        if f == "ndpointer":
            flags = []
            for kw in node.keywords:
                if kw.arg == "flags":
                    flags = [e.value for e in kw.value.elts]
            return {"kind": "ndpointer", "dtype": _type(node.args[0])["name"], "flags": flags}
    raise ValueError(f"unhandled type expression at line {node.lineno}: {ast.dump(node)}")


def extract(path):
    tree = ast.parse(open(path).read())
    structs, funcs = {}, {}
    for node in ast.walk(tree):
        if isinstance(node, ast.ClassDef) and any(isinstance(b, ast.Name) and b.id == "Structure" for b in node.bases):
            for st in node.body:
                if isinstance(st, ast.Assign) and st.targets[0].id == "_fields_":
                    structs[node.name] = {"line": node.lineno,
                                          "fields": [[e.elts[0].value, e.elts[1].id] for e in st.value.elts]}
        if isinstance(node, ast.Assign) and len(node.targets) == 1:
            t = node.targets[0]
            # self.lib.<symbol>.argtypes / .restype
            if (isinstance(t, ast.Attribute) and t.attr in ("argtypes", "restype")
                    and isinstance(t.value, ast.Attribute) and isinstance(t.value.value, ast.Attribute)
                    and t.value.value.attr == "lib"):
                sym = t.value.attr
                f = funcs.setdefault(sym, {})
                if t.attr == "argtypes":
                    f["argtypes"] = [_type(e) for e in node.value.elts]
                    f["line"] = node.lineno
                else:
                    f["restype"] = _type(node.value)
    return {"source": REL.replace(os.sep, "/"), "structures": structs,
            "functions": dict(sorted(funcs.items()))}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--check", action="store_true")
    args = ap.parse_args()
    ref = os.environ.get("SFD_REFERENCE_DIR")
    if not ref:
        sys.exit("set SFD_REFERENCE_DIR to the reference checkout")
    spec = extract(os.path.join(ref, REL))
    if args.check:
        with open(OUT) as f:
            same = json.load(f) == spec
        print("fixture matches" if same else "fixture differs")
        sys.exit(0 if same else 1)
    with open(OUT, "w") as f:
        json.dump(spec, f, indent=1)
    print(f"{len(spec['functions'])} functions, {len(spec['structures'])} structures -> {OUT}")


if __name__ == "__main__":
    main()
