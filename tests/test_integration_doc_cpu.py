"""The ctypes stub that INTEGRATION.md gives a DeepDRR maintainer must lay out drr_project_args
exactly as include/drr_gb300.h does, and so must the package's own binding (deepdrr_gb300/_lib.py):
a binding that is missing fields would have the library read past the caller's struct. The
library also checks struct_size, and says its own size when it does not match."""
import ast
import ctypes
import re
from pathlib import Path

from deepdrr_gb300 import _lib

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "drr_gb300.h"
DOC = ROOT / "INTEGRATION.md"

C_TYPES = {"uint32_t": ctypes.c_uint32, "int32_t": ctypes.c_int32, "float": ctypes.c_float,
           "double": ctypes.c_double, "uint8_t": ctypes.c_uint8, "int8_t": ctypes.c_int8}


def header_struct(name):
    """(field, ctypes type) of `typedef struct { ... } name;` in the header; pointers are c_void_p."""
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    m = re.search(r"typedef struct \{([^{}]*)\}\s*" + name + ";", text)
    assert m, name
    fields = []
    for decl in m.group(1).split(";"):
        decl = " ".join(decl.split())
        if not decl:
            continue
        decl = decl.replace("const ", "")
        base, rest = decl.split(" ", 1)
        for item in rest.split(","):
            item = item.strip()
            arr = re.match(r"(\w+)\[(\d+)\]$", item)
            if item.startswith("*"):
                fields.append((item.lstrip("*"), ctypes.c_void_p))
            elif arr:
                fields.append((arr.group(1), C_TYPES[base] * int(arr.group(2))))
            else:
                fields.append((item, C_TYPES[base]))
    return fields


def doc_classes():
    """The ctypes Structure classes of INTEGRATION.md's binding, defined without running the rest
    of the snippet."""
    blocks = re.findall(r"```python\n(.*?)```", DOC.read_text(), flags=re.S)
    src = next(b for b in blocks if "class drr_project_args" in b)
    tree = ast.parse(src)
    ns = {"ctypes": ctypes}
    for node in tree.body:
        if isinstance(node, ast.ClassDef):
            exec(compile(ast.Module([node], []), "INTEGRATION.md", "exec"), ns)
    return ns


def layout(cls):
    return [(name, getattr(cls, name).offset, getattr(cls, name).size) for name, _ in cls._fields_]


def test_package_binding_matches_the_header():
    for name in ("drr_project_args", "drr_adjoint_args", "drr_volume_desc", "drr_mesh_desc", "drr_tune_result"):
        hdr = header_struct(name)
        ours = getattr(_lib, name)._fields_
        assert [f for f, _ in ours] == [f for f, _ in hdr], name
        for (f, t_ours), (_, t_hdr) in zip(ours, hdr):
            assert ctypes.sizeof(t_ours) == ctypes.sizeof(t_hdr), (name, f)


def test_documented_stub_matches_the_package_binding():
    ns = doc_classes()
    for name in ("drr_project_args", "drr_volume_desc"):
        assert layout(ns[name]) == layout(getattr(_lib, name)), name
        assert ctypes.sizeof(ns[name]) == ctypes.sizeof(getattr(_lib, name)), name


def test_library_rejects_a_struct_of_another_size_before_reading_it():
    lib = _lib.load()
    args = _lib.drr_project_args()
    assert args.struct_size == ctypes.sizeof(_lib.drr_project_args)
    args.struct_size = ctypes.sizeof(_lib.drr_project_args) - 24  # a binding without the last four fields
    assert lib.drr_project(None, None, ctypes.byref(args), None) == _lib.DRR_ERR_INVALID_ARGUMENT
    msg = lib.drr_last_error().decode()
    assert "struct_size" in msg
    assert int(re.search(r"has (\d+) bytes", msg).group(1)) == ctypes.sizeof(_lib.drr_project_args)
    for fn in (lambda: lib.drr_graph_create(None, None, ctypes.byref(args), ctypes.byref(ctypes.c_void_p())),
               lambda: lib.drr_autotune(None, None, ctypes.byref(args), 1, None, ctypes.byref(_lib.drr_tune_result()))):
        assert fn() == _lib.DRR_ERR_INVALID_ARGUMENT
        assert "struct_size" in lib.drr_last_error().decode()
    args.struct_size = ctypes.sizeof(_lib.drr_project_args)
    adj = _lib.drr_adjoint_args()
    adj.struct_size = 8
    assert lib.drr_project_adjoint(None, None, ctypes.byref(args), ctypes.byref(adj), None) == \
        _lib.DRR_ERR_INVALID_ARGUMENT
    assert "adj->struct_size" in lib.drr_last_error().decode()
    # with both sizes right, the NULL handles are what is rejected
    adj.struct_size = ctypes.sizeof(_lib.drr_adjoint_args)
    assert lib.drr_project_adjoint(None, None, ctypes.byref(args), ctypes.byref(adj), None) == \
        _lib.DRR_ERR_INVALID_ARGUMENT
    assert "NULL" in lib.drr_last_error().decode()
