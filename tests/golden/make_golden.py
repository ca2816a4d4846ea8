"""Extract golden vectors from the reference's own test files (read as text).

The reference (exponax 0.2.0) needs JAX, which is not importable here, so its
tests cannot run.  Their literal expected values are still the best pin for
the oracle: this script parses the test sources with ``ast`` and writes the
expected arrays/tuples to ``tests/golden/*.json``.  Nothing from the
reference is executed; only literal expressions (lists, ``slice(...)`` and
integer arithmetic) are evaluated.

Usage (only where the reference tree is mounted):
    python tests/golden/make_golden.py /root/reference
"""

import ast
import json
import os
import sys


def _literal(node, src):
    """Evaluate a literal expression (lists, tuples, True/False, ints,
    slice(...), +,-,//) without executing any reference code."""
    code = ast.get_source_segment(src, node)
    tree = ast.parse(code, mode="eval")
    allowed = (ast.Expression, ast.List, ast.Tuple, ast.Constant, ast.Call, ast.Name, ast.Load,
               ast.BinOp, ast.UnaryOp, ast.Add, ast.Sub, ast.FloorDiv, ast.USub, ast.Mult)
    for n in ast.walk(tree):
        if not isinstance(n, allowed):
            raise ValueError(f"non-literal node {type(n).__name__} in {code[:60]}")
        if isinstance(n, ast.Name) and n.id not in ("slice", "None", "True", "False"):
            raise ValueError(f"unexpected name {n.id}")
        if isinstance(n, ast.Call) and not (isinstance(n.func, ast.Name) and n.func.id == "slice"):
            raise ValueError("only slice() calls are allowed")
    return eval(compile(tree, "<golden>", "eval"), {"__builtins__": {}}, {"slice": slice, "None": None})


def _call_name(call):
    f = call.func
    parts = []
    while isinstance(f, ast.Attribute):
        parts.append(f.attr)
        f = f.value
    if isinstance(f, ast.Name):
        parts.append(f.id)
    return ".".join(reversed(parts))


def extract_masks(path):
    src = open(path).read()
    out = []
    for node in ast.walk(ast.parse(src)):
        if not (isinstance(node, ast.Call) and _call_name(node).endswith("testing.assert_equal")):
            continue
        got, exp = node.args
        fn = _call_name(got).split(".")[-1]
        args = [_literal(a, src) for a in got.args]
        kwargs = {k.arg: _literal(k.value, src) for k in got.keywords}
        name = _call_name(exp)
        if name.endswith("ones"):
            # np.ones(shape, dtype=bool): store the all-True array by shape
            shape = _literal(exp.args[0], src)
            expected = {"ones_shape": list(shape)}
        else:
            assert name.endswith("array"), name
            expected = _literal(exp.args[0], src)
        out.append({"fn": fn, "args": args, "kwargs": kwargs, "expected": expected,
                    "line": node.lineno})
    return out


def _slices_to_json(t):
    return [[[s.start, s.stop, s.step] for s in block] for block in t]


def extract_mode_slices(path):
    src = open(path).read()
    out = []
    for node in ast.walk(ast.parse(src)):
        if not isinstance(node, ast.Assert):
            continue
        t = node.test
        if not (isinstance(t, ast.Compare) and isinstance(t.left, ast.Call)):
            continue
        if not _call_name(t.left).endswith("get_modes_slices"):
            continue
        args = [_literal(a, src) for a in t.left.args]
        expected = _literal(t.comparators[0], src)
        out.append({"args": args, "expected": _slices_to_json(expected), "line": node.lineno})
    return out


def main(ref_root):
    here = os.path.dirname(os.path.abspath(__file__))
    masks = extract_masks(os.path.join(ref_root, "tests", "test_filter_masks.py"))
    slices = extract_mode_slices(os.path.join(ref_root, "tests", "test_mode_slices_generation.py"))
    with open(os.path.join(here, "filter_masks.json"), "w") as f:
        json.dump({"source": "exponax tests/test_filter_masks.py", "cases": masks}, f)
    with open(os.path.join(here, "mode_slices.json"), "w") as f:
        json.dump({"source": "exponax tests/test_mode_slices_generation.py", "cases": slices}, f)
    print(f"{len(masks)} mask cases, {len(slices)} mode-slice cases")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
