"""The Julia binding (julia/NBodySimulatorGPU.jl) against the C header it
binds: every struct it passes to libnbg has the C layout field for field
(names, order, offsets and sizes computed by Julia's C-compatible layout
rules, compared with gcc's offsetof on include/nbg.h), and every ccall names
a function the header declares with its number of parameters. Julia itself
is not installed here, so this is the binding's check."""
import os
import re
import subprocess
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
JL = os.path.join(ROOT, "julia", "NBodySimulatorGPU.jl")
HDR = os.path.join(ROOT, "include", "nbg.h")

# size and alignment of the Julia field types the binding uses (C layout)
JL_TYPES = {"Int32": (4, 4), "UInt32": (4, 4), "Int64": (8, 8), "UInt64": (8, 8), "Float64": (8, 8),
            "Ptr{Float64}": (8, 8), "NTuple{6, Float64}": (48, 8)}
# the C declaration each Julia type stands for
C_OF_JL = {"Int32": "int32_t", "UInt32": "uint32_t", "Int64": "int64_t", "UInt64": "uint64_t",
           "Float64": "double", "Ptr{Float64}": "const double*", "NTuple{6, Float64}": "double[6]"}
STRUCTS = {"NbgSystemDesc": "nbg_system_desc", "NbgRunStats": "nbg_run_stats", "NbgEnergies": "nbg_energies",
           "NbgRespaStats": "nbg_respa_stats"}


def _julia_struct(text, name):
    m = re.search(r"(?:mutable\s+)?struct\s+" + name + r"\s*\n(.*?)\nend", text, re.S)
    assert m, name
    fields = []
    for line in m.group(1).splitlines():
        line = line.split("#")[0].strip()
        if line:
            f, t = line.split("::")
            fields.append((f.strip(), t.strip()))
    return fields


def _c_struct(text, name):
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    m = re.search(r"typedef struct " + name + r"\s*\{(.*?)\}\s*" + name + ";", text, re.S)
    assert m, name
    fields = []
    for decl in m.group(1).split(";"):
        decl = " ".join(decl.split())
        if not decl:
            continue
        m2 = re.match(r"((?:const\s+)?\w+\s*\*?)\s*(.*)", decl)
        base = m2.group(1).replace(" ", "").replace("const", "const ")
        for nm in m2.group(2).split(","):
            nm = nm.strip()
            arr = re.match(r"(\w+)\[(\d+)\]", nm)
            if arr:
                fields.append((arr.group(1), f"{base}[{arr.group(2)}]"))
            else:
                ptr = nm.startswith("*")
                fields.append((nm.lstrip("*"), base + ("*" if ptr else "")))
    return fields


def _julia_layout(fields):
    off, out, align = 0, [], 1
    for f, t in fields:
        size, a = JL_TYPES[t]
        off = (off + a - 1) // a * a
        out.append((f, off, size))
        off += size
        align = max(align, a)
    return out, (off + align - 1) // align * align


def _c_offsets(struct, fields):
    lines = [f'printf("%zu %zu\\n", offsetof({struct}, {f}), sizeof((({struct}*)0)->{f}));' for f, _ in fields]
    src = ('#include <stddef.h>\n#include <stdio.h>\n#include "nbg.h"\nint main(void) {\n'
           + "\n".join(lines) + f'\nprintf("%zu\\n", sizeof({struct}));\nreturn 0; }}\n')
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "t")
        subprocess.run(["gcc", "-I", os.path.dirname(HDR), c, "-o", exe], check=True)
        vals = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    pairs = [(int(vals[2 * k]), int(vals[2 * k + 1])) for k in range(len(fields))]
    return pairs, int(vals[-1])


def test_julia_structs_have_the_c_layout():
    jl, hdr = open(JL).read(), open(HDR).read()
    for jname, cname in STRUCTS.items():
        jf = _julia_struct(jl, jname)
        cf = _c_struct(hdr, cname)
        assert [f for f, _ in jf] == [f for f, _ in cf], jname
        for (f, jt), (_, ct) in zip(jf, cf):
            assert C_OF_JL[jt] == ct, (jname, f, jt, ct)
        layout, jsize = _julia_layout(jf)
        coffs, csize = _c_offsets(cname, cf)
        assert [(o, s) for _, o, s in layout] == coffs, jname
        assert jsize == csize, jname


def _ccalls(text):
    out = []
    for m in re.finditer(r"@ccall\(?\s*libnbg\.(nbg_\w+)\(", text):
        depth, k = 1, m.end()
        while depth:
            depth += {"(": 1, ")": -1}.get(text[k], 0)
            k += 1
        args = text[m.end():k - 1]
        depth, n, cur = 0, 0, ""
        for ch in args:
            depth += {"(": 1, ")": -1, "{": 1, "}": -1}.get(ch, 0)
            if ch == "," and depth == 0:
                n += 1
                cur = ""
            else:
                cur += ch
        n += 1 if cur.strip() else 0
        out.append((m.group(1), n))
    return out


def _c_prototypes(text):
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    protos = {}
    for m in re.finditer(r"NBG_API[^;(]*?\b(nbg_\w+)\s*\(([^)]*)\)\s*;", text, re.S):
        params = m.group(2).strip()
        protos[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    return protos


def test_every_ccall_matches_a_header_prototype():
    calls = _ccalls(open(JL).read())
    protos = _c_prototypes(open(HDR).read())
    names = {n for n, _ in calls}
    # the binding covers the drop-in, the loop, checkpoints, energies, rdf and the learned add-on
    for need in ("nbg_create", "nbg_destroy", "nbg_accel", "nbg_run", "nbg_energy", "nbg_rdf_histogram",
                 "nbg_get_step", "nbg_set_step", "nbg_last_error", "nbg_respa_run", "nbg_ml_train"):
        assert need in names, need
    for n, k in calls:
        assert n in protos, n
        assert protos[n] == k, (n, k, protos[n])
