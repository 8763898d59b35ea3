"""Load the reference's Python modules with Taichi's source transformation restated.

Test infrastructure only (golden-vector generation in this container).  Taichi compiles a
kernel from its Python AST; the two rewrites below are the parts of that transformation the
particle-flow-map step depends on and plain Python cannot express:

* ``int(x)`` on a Taichi vector truncates elementwise, so every call to the builtin ``int``
  becomes ``_ti_int(x)``;
* ``ti.atomic_<op>(F[idx], v)`` updates the field element in place, so it becomes
  ``_ti_atomic("<op>", F, idx, v)``.

Everything else in the reference source runs unmodified against ``oracle/ref_shim/taichi``.
"""
import ast
import importlib.abc
import importlib.util
import os
import sys
import types

SHIM_DIR = os.path.dirname(os.path.abspath(__file__))


class _TaichiRewrite(ast.NodeTransformer):
    def visit_Call(self, node):
        self.generic_visit(node)
        if isinstance(node.func, ast.Name) and node.func.id == "int" and len(node.args) == 1:
            node.func = ast.Name(id="_ti_int", ctx=ast.Load())
            return node
        f = node.func
        if (isinstance(f, ast.Attribute) and isinstance(f.value, ast.Name) and f.value.id == "ti"
                and f.attr.startswith("atomic_") and len(node.args) == 2
                and isinstance(node.args[0], ast.Subscript)):
            target = node.args[0]
            new = ast.Call(
                func=ast.Name(id="_ti_atomic", ctx=ast.Load()),
                args=[ast.Constant(f.attr[len("atomic_"):]), target.value,
                      target.slice, node.args[1]],
                keywords=[])
            return ast.copy_location(new, node)
        return node


class _RefFinder(importlib.abc.MetaPathFinder, importlib.abc.Loader):
    def __init__(self, ref_dir, names):
        self.ref_dir = ref_dir
        self.names = set(names)

    def find_spec(self, fullname, path, target=None):
        if fullname in self.names:
            return importlib.util.spec_from_loader(fullname, self)
        return None

    def create_module(self, spec):
        return None

    def exec_module(self, module):
        import taichi  # the shim
        path = os.path.join(self.ref_dir, module.__name__ + ".py")
        src = open(path).read()
        tree = _TaichiRewrite().visit(ast.parse(src, filename=path))
        ast.fix_missing_locations(tree)
        module.__file__ = path
        module.__dict__["_ti_int"] = taichi._ti_int
        module.__dict__["_ti_atomic"] = taichi._ti_atomic
        exec(compile(tree, path, "exec"), module.__dict__)


def install(ref_dir, names, hyperparameters, stubs=None):
    """Make ``names`` (reference modules in ``ref_dir``) importable through the rewrite.

    ``hyperparameters`` is a dict that becomes the ``hyperparameters`` module the reference
    star-imports; ``stubs`` maps module names to dicts for modules that are not installed here
    (matplotlib/vtk writers, the 2D driver's missing ``single_vortex``).
    """
    if SHIM_DIR not in sys.path:
        sys.path.insert(0, SHIM_DIR)
    for n in list(names) + ["hyperparameters"] + list((stubs or {}).keys()):
        sys.modules.pop(n, None)
    hp = types.ModuleType("hyperparameters")
    hp.__dict__.update(hyperparameters)
    sys.modules["hyperparameters"] = hp
    for name, attrs in (stubs or {}).items():
        m = types.ModuleType(name)
        m.__dict__.update(attrs)
        sys.modules[name] = m
    for f in list(sys.meta_path):
        if isinstance(f, _RefFinder):
            sys.meta_path.remove(f)
    finder = _RefFinder(ref_dir, names)
    sys.meta_path.insert(0, finder)
    return finder
