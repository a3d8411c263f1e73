"""bench.py: every name a function reads is defined (a parameter, a local, a
module-level name or a builtin).  bench.py needs a GPU to run, so this catches
a misspelt or out-of-scope name on CPU before a GPU run does."""
import ast
import builtins
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _undefined_names(src):
    tree = ast.parse(src)
    module = set()
    for node in tree.body:
        if isinstance(node, (ast.FunctionDef, ast.ClassDef)):
            module.add(node.name)
        elif isinstance(node, (ast.Import, ast.ImportFrom)):
            module.update((a.asname or a.name).split(".")[0] for a in node.names)
        elif isinstance(node, (ast.Assign, ast.AnnAssign)):
            targets = node.targets if isinstance(node, ast.Assign) else [node.target]
            for t in targets:
                module.update(n.id for n in ast.walk(t) if isinstance(n, ast.Name))
    bad = []
    for fn in (n for n in tree.body if isinstance(n, ast.FunctionDef)):
        defined = {a.arg for a in fn.args.args + fn.args.kwonlyargs}
        for n in ast.walk(fn):
            if isinstance(n, ast.Name) and isinstance(n.ctx, (ast.Store, ast.Del)):
                defined.add(n.id)
            elif isinstance(n, (ast.FunctionDef, ast.Lambda)) and n is not fn:
                defined.update(a.arg for a in n.args.args + n.args.kwonlyargs)
                if isinstance(n, ast.FunctionDef):
                    defined.add(n.name)
            elif isinstance(n, (ast.Import, ast.ImportFrom)):
                defined.update((a.asname or a.name).split(".")[0] for a in n.names)
            elif isinstance(n, ast.ExceptHandler) and n.name:
                defined.add(n.name)
        for n in ast.walk(fn):
            if isinstance(n, ast.Name) and isinstance(n.ctx, ast.Load):
                if n.id not in defined and n.id not in module and not hasattr(builtins, n.id):
                    bad.append((fn.name, n.id, n.lineno))
    return bad


def test_bench_functions_read_only_defined_names():
    with open(os.path.join(ROOT, "bench.py")) as f:
        assert _undefined_names(f.read()) == []


def test_checker_finds_an_undefined_name():
    assert _undefined_names("def f(a):\n    return a + b\n") == [("f", "b", 2)]
