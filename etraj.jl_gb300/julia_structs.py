"""Julia mirrors of the C ABI's structs, generated from include/etraj.h.

The `ccall` binding of eTraj.jl (the `solver=:cuda` keyword) passes an
`etraj_job` and an `etraj_result` by reference, so its Julia structs must have
the C layout field for field.  `julia_structs()` writes them from the header's
`typedef struct` blocks (C field names, C order; fixed arrays become NTuples,
pointers Ptr{Float64}); `julia_layout()` gives each field's offset and each
struct's size under the C alignment rules, which Julia applies to isbits
structs, so a test can hold them against the compiler's own offsetof.

python -m etraj_gb300.julia_structs   prints the Julia definitions.
"""
import os
import re

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "etraj.h")

# C struct -> Julia struct, in dependency order
STRUCTS = [("etraj_mono_laser", "CMono"), ("etraj_laser", "CLaser"), ("etraj_target", "CTarget"),
           ("etraj_job", "CJob"), ("etraj_result", "CResult")]
MUTABLE = {"CResult"}  # filled in by the library through Ref
SCALARS = {"int32_t": ("Int32", 4), "int64_t": ("Int64", 8), "uint64_t": ("UInt64", 8), "double": ("Float64", 8)}


def parse_header(path=HEADER):
    """{c_name: [(field, c_type, count, is_pointer)]} of the header's typedef structs."""
    text = re.sub(r"/\*.*?\*/", "", open(path).read(), flags=re.S)
    out = {}
    for body, name in re.findall(r"typedef\s+struct\s+\w*\s*\{(.*?)\}\s*(\w+)\s*;", text, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            m = re.match(r"(?:const\s+)?(\w+)\s*(.*)$", decl)
            ctype, rest = m.group(1), m.group(2)
            for d in rest.split(","):
                d = d.strip()
                ptr = d.startswith("*")
                d = d.lstrip("*").strip()
                a = re.match(r"(\w+)\s*(?:\[(\d+)\])?$", d)
                fields.append((a.group(1), ctype, int(a.group(2) or 1), ptr))
        out[name] = fields
    return out


def _jl_type(ctype, count, ptr, names):
    if ptr:
        base, size, align = "Ptr{Float64}", 8, 8
    elif ctype in SCALARS:
        base, size = SCALARS[ctype]
        align = size
    else:
        base = names[ctype]
        size, align = None, None  # nested struct: filled by the caller
    return base, size, align


def julia_layout(path=HEADER):
    """{c_name: (size, {field: offset})} under C's (and Julia's isbits) alignment rules."""
    parsed = parse_header(path)
    names = dict(STRUCTS)
    done = {}
    for cname, _ in STRUCTS:
        off, max_align, offs = 0, 1, {}
        for field, ctype, count, ptr in parsed[cname]:
            base, size, align = _jl_type(ctype, count, ptr, names)
            if size is None:
                size, align = done[ctype][0], done[ctype][2]
            off = (off + align - 1) // align * align
            offs[field] = off
            off += size * count
            max_align = max(max_align, align)
        size = (off + max_align - 1) // max_align * max_align
        done[cname] = (size, offs, max_align)
    return {k: (v[0], v[1]) for k, v in done.items()}


def julia_structs(path=HEADER):
    """The Julia struct definitions, one per C struct, C field names in C order."""
    parsed = parse_header(path)
    names = dict(STRUCTS)
    lines = []
    for cname, jname in STRUCTS:
        fields = []
        for field, ctype, count, ptr in parsed[cname]:
            base = _jl_type(ctype, count, ptr, names)[0]
            t = base if count == 1 else "NTuple{%d,%s}" % (count, base)
            fields.append("%s::%s" % (field, t))
        head = ("mutable struct " if jname in MUTABLE else "struct ") + jname
        # a few fields per line, as the binding is written
        row, rows = [], []
        for f in fields:
            if row and len("; ".join(row + [f])) > 96:
                rows.append(row)
                row = []
            row.append(f)
        rows.append(row)
        pad = " " * (len(head) + 2)
        text = head + "; " + "; ".join(rows[0])
        for r in rows[1:]:
            text += "\n" + pad + "; ".join(r)
        lines.append(text + "; end")
    return "\n".join(lines)


if __name__ == "__main__":
    print(julia_structs())
