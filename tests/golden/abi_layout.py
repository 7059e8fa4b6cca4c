"""ABI layout of a cubbs_bbs_gpu_abi.h: every struct's sizeof and field
offsets, every #define constant and every function prototype, measured by
compiling the header with the host C compiler.

Used by make_abi_layout.py (on the reference header, to write
abi_layout.json) and by tests/test_abi_layout.py (on this repository's
header, to compare)."""
import json
import pathlib
import re
import subprocess
import tempfile

STRUCT_RE = re.compile(r"typedef\s+struct\s+(\w+)\s*\{(.*?)\}\s*(\w+)\s*;", re.S)
DEFINE_RE = re.compile(r"^#define\s+(CUBBS_\w+)\s+(\d+)u?\s*$", re.M)
PROTO_RE = re.compile(r"\b(int32_t\s+(cubbs_bbs_gpu_\w+)\s*\(([^;{]*?)\))\s*;", re.S)


def _strip_comments(text: str) -> str:
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    return re.sub(r"//[^\n]*", " ", text)


def parse(header_text: str):
    text = _strip_comments(header_text)
    structs = {}
    for m in STRUCT_RE.finditer(text):
        name = m.group(3)
        fields = []
        for decl in m.group(2).split(";"):
            decl = decl.strip()
            if not decl:
                continue
            f = re.search(r"(\w+)\s*(\[[^\]]*\])?\s*$", decl)
            fields.append(f.group(1))
        structs[name] = fields
    defines = {m.group(1): int(m.group(2)) for m in DEFINE_RE.finditer(text)}
    protos = {m.group(2): " ".join(m.group(1).split()) for m in PROTO_RE.finditer(text)}
    return structs, defines, protos


def measure(header: pathlib.Path, structs, cc: str = "gcc"):
    """sizeof / offsetof of every struct and field, compiled against `header`."""
    lines = ["#include <stddef.h>", "#include <stdio.h>", f'#include "{header.resolve()}"', "int main(void) {",
             '  printf("{");']
    first = True
    for name, fields in structs.items():
        sep = "" if first else ","
        first = False
        lines.append(f'  printf("{sep}\\"{name}\\": {{\\"size\\": %zu, \\"align\\": %zu", sizeof({name}), '
                     f'_Alignof({name}));')
        for fld in fields:
            lines.append(f'  printf(", \\"{fld}\\": %zu", offsetof({name}, {fld}));')
        lines.append('  printf("}");')
    lines += ['  printf("}\\n");', "  return 0;", "}"]
    with tempfile.TemporaryDirectory() as d:
        src = pathlib.Path(d) / "layout.c"
        exe = pathlib.Path(d) / "layout"
        src.write_text("\n".join(lines) + "\n")
        subprocess.run([cc, "-std=c11", "-O0", "-o", str(exe), str(src)], check=True, capture_output=True)
        out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return json.loads(out)


def check_prototypes(header: pathlib.Path, protos, cc: str = "gcc"):
    """Compiles, against `header`, one function pointer per prototype typed by
    the given prototype text and initialised with the header's function; a
    parameter or return type that differs fails the compile.  Returns
    (ok, compiler output)."""
    lines = [f'#include "{header.resolve()}"']
    for name, proto in protos.items():
        ptr = proto.replace(name, f"(*chk_{name})", 1)
        lines.append(f"{ptr} = {name};")
    with tempfile.TemporaryDirectory() as d:
        src = pathlib.Path(d) / "protos.c"
        src.write_text("\n".join(lines) + "\nint main(void) { return 0; }\n")
        res = subprocess.run([cc, "-std=c11", "-Werror=incompatible-pointer-types", "-c", "-o",
                              str(pathlib.Path(d) / "protos.o"), str(src)], capture_output=True, text=True)
    return res.returncode == 0, res.stderr
