"""Extracts the known-answer vectors of pjz's own tests into JSON.

The reference (pjz) needs JAX, which cannot be imported here, so its test
files are read as text: every literal argument of the assertions in
``tests/test_boundaries.py``, ``tests/test_frequencies.py`` and
``tests/test_waveforms.py``, and every ``parametrize`` table of
``tests/test_layers.py`` (epsilon rendering; its expected values include
arithmetic such as ``9 / 4``, evaluated here), is pulled out with ``ast`` and
written, with its source line, to ``reference_kats.json`` beside this
script.  Run it from the
repository root with the reference checkout's path as the only argument.
"""

import ast
import json
import os
import sys


def _literal(node):
  try:
    return ast.literal_eval(node)
  except ValueError:
    return None


def _number(node):
  """Value of a literal built from numbers, tuples and + - * / (the
  expected values of the layer tests)."""
  if isinstance(node, ast.Constant) and isinstance(node.value, (int, float)):
    return node.value
  if isinstance(node, (ast.Tuple, ast.List)):
    return [_number(e) for e in node.elts]
  if isinstance(node, ast.UnaryOp) and isinstance(node.op, (ast.USub, ast.UAdd)):
    v = _number(node.operand)
    return -v if isinstance(node.op, ast.USub) else v
  if isinstance(node, ast.BinOp):
    a, b = _number(node.left), _number(node.right)
    ops = {ast.Add: lambda: a + b, ast.Sub: lambda: a - b,
           ast.Mult: lambda: a * b, ast.Div: lambda: a / b}
    return ops[type(node.op)]()
  raise ValueError(f"not a numeric literal: {ast.unparse(node)}")


def _parametrize_tables(fn):
  """[(argument names, rows)] of a test function's parametrize decorators;
  a ``pytest.param(..., id=...)`` row keeps its id."""
  out = []
  for dec in fn.decorator_list:
    if not (isinstance(dec, ast.Call) and ast.unparse(dec.func).endswith("parametrize")):
      continue
    names = [n.strip() for n in dec.args[0].value.split(",")]
    rows = []
    for e in dec.args[1].elts:
      if isinstance(e, ast.Call):  # pytest.param(values..., id=...)
        vals = [_number(a) for a in e.args]
        rid = {k.arg: k.value.value for k in e.keywords}.get("id")
      else:
        vals, rid = _number(e), None
      rows.append({"values": vals, "id": rid, "line": e.lineno})
    out.append({"names": names, "rows": rows})
  return out


def _calls(tree):
  for node in ast.walk(tree):
    if isinstance(node, ast.Call):
      yield node


def _kw(call):
  return {k.arg: _literal(k.value) for k in call.keywords}


def extract(ref_root):
  tests = os.path.join(ref_root, "tests")
  kats = {"source": "pjz tests (read as text)", "cases": []}

  path = os.path.join(tests, "test_boundaries.py")
  tree = ast.parse(open(path).read())
  for call in _calls(tree):
    name = ast.unparse(call.func)
    if name.endswith("assert_array_equal"):
      target = ast.unparse(call.args[0])
      kats["cases"].append({
          "file": "tests/test_boundaries.py", "line": call.lineno,
          "kind": "absorption_mask", "index": target,
          "expected": _literal(call.args[1])})
    if name.endswith("assert_array_almost_equal"):
      inner = call.args[0]
      kats["cases"].append({
          "file": "tests/test_boundaries.py", "line": call.lineno,
          "kind": "pml_sigma", "kwargs": _kw(inner),
          "expected": _literal(call.args[1])})
  for call in _calls(tree):
    if ast.unparse(call.func).endswith("absorption_mask"):
      for c in kats["cases"]:
        if c["kind"] == "absorption_mask":
          c["kwargs"] = _kw(call)

  path = os.path.join(tests, "test_frequencies.py")
  src = open(path).read()
  tree = ast.parse(src)
  for fn in tree.body:
    if isinstance(fn, ast.FunctionDef):
      kats["cases"].append({
          "file": "tests/test_frequencies.py", "line": fn.lineno,
          "kind": fn.name, "source": ast.get_source_segment(src, fn)})

  path = os.path.join(tests, "test_waveforms.py")
  src = open(path).read()
  tree = ast.parse(src)
  for call in _calls(tree):
    if ast.unparse(call.func).endswith("ramped_sin"):
      kats["cases"].append({
          "file": "tests/test_waveforms.py", "line": call.lineno,
          "kind": "ramped_sin", "kwargs": _kw(call),
          "args": [ast.unparse(a) for a in call.args]})

  path = os.path.join(tests, "test_layers.py")
  tree = ast.parse(open(path).read())
  for fn in tree.body:
    if isinstance(fn, ast.FunctionDef):
      tables = _parametrize_tables(fn)
      if tables:
        kats["cases"].append({
            "file": "tests/test_layers.py", "line": fn.lineno,
            "kind": "render_" + fn.name[len("test_"):], "tables": tables})
  return kats


if __name__ == "__main__":
  ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
  out = os.path.join(os.path.dirname(os.path.abspath(__file__)),
                     "reference_kats.json")
  with open(out, "w") as f:
    json.dump(extract(ref), f, indent=1)
  print("wrote", out)
