"""Generate tests/golden/struct_layouts.json from the reference's own headers.

Run from the repo root in a container that has the reference project at
/root/reference (the output is committed; the tests only read the JSON).

For each of the four structs the drop-in boundary must match byte for byte,
a probe program is compiled with the reference's definition and prints
sizeof and every member's offsetof:

  * sylver_inform_t, sylver_options_t: the probe includes the reference's C
    header include/sylver/sylver.h as it is (C, gcc);
  * options_c, inform_c: they live in src/sylver_ciface.hxx, which includes
    SPRAL headers that are absent.  The generator takes the member lines of
    the two struct bodies out of that file (member functions and default
    initialisers dropped) into a temporary probe, with the reference's
    enum types (sylver::PivotMethod, FailedPivotMethod, CPUTopology, Flag,
    all declared `: int`) written as int, which has the same size and
    alignment.  Nothing of the reference is written into this repository
    except the numbers.
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import sys
import tempfile

REF = "/root/reference"
HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "struct_layouts.json")


def c_members(body: str):
    """(type, name) of the data members of a C/C++ struct body."""
    out = []
    for line in body.splitlines():
        line = re.sub(r"//.*", "", line).strip()
        if not line or "(" in line or line.startswith(("using", "}", "{")):
            continue
        m = re.match(r"^([\w:]+(?:\s+[\w:]+)*)\s+(\w+)\s*(\[\s*\d+\s*\])?\s*(=[^;]*)?;$", line)
        if m:
            out.append((m.group(1), m.group(2) + (m.group(3) or "")))
    return out


def struct_body(txt: str, head: str) -> str:
    i = txt.index(head)
    j = txt.index("{", i)
    depth, k = 0, j
    while True:
        if txt[k] == "{":
            depth += 1
        elif txt[k] == "}":
            depth -= 1
            if depth == 0:
                return txt[j + 1:k]
        k += 1


def probe(src: str, cc: str, flags) -> dict:
    with tempfile.TemporaryDirectory() as d:
        f = os.path.join(d, "p." + ("c" if cc == "gcc" else "cpp"))
        open(f, "w").write(src)
        exe = os.path.join(d, "p")
        subprocess.run([cc, *flags, f, "-o", exe], check=True)
        return json.loads(subprocess.run([exe], capture_output=True, text=True,
                                         check=True).stdout)


def printer(name: str, ctype: str, members) -> str:
    parts = [f'printf("\\"{name}\\": {{\\"sizeof\\": %zu", sizeof({ctype}));']
    for _, m in members:
        m = m.split("[")[0]
        parts.append(f'printf(", \\"{m}\\": %zu", offsetof({ctype}, {m}));')
    parts.append('printf("}");')
    return "\n".join(parts)


def main():
    hdr = os.path.join(REF, "include", "sylver", "sylver.h")
    htxt = open(hdr).read()
    inf = c_members(struct_body(htxt, "typedef struct {"))
    opt_head = htxt.index("typedef struct {", htxt.index("sylver_inform_t"))
    opt = c_members(struct_body(htxt[opt_head:], "typedef struct {"))
    src1 = "#include <stddef.h>\n#include <stdio.h>\n#include \"%s\"\nint main(void){\n" % hdr
    src1 += 'printf("{");\n' + printer("sylver_inform_t", "sylver_inform_t", inf)
    src1 += 'printf(", ");\n' + printer("sylver_options_t", "sylver_options_t", opt)
    src1 += 'printf("}\\n"); return 0;}\n'
    a = probe(src1, "gcc", [])

    ctxt = open(os.path.join(REF, "src", "sylver_ciface.hxx")).read()
    oc = c_members(struct_body(ctxt, "struct options_c"))
    ic = c_members(struct_body(ctxt, "struct inform_c"))

    def as_int(t):
        return "int" if ("sylver::" in t or t == "Flag") else t
    decl = "struct options_c {\n" + "".join(f"  {as_int(t)} {m};\n" for t, m in oc) + "};\n"
    decl += "struct inform_c {\n" + "".join(f"  {as_int(t)} {m};\n" for t, m in ic) + "};\n"
    src2 = "#include <cstddef>\n#include <cstdio>\n" + decl + "int main(){\n"
    src2 += 'printf("{");\n' + printer("options_c", "options_c", oc)
    src2 += 'printf(", ");\n' + printer("inform_c", "inform_c", ic)
    src2 += 'printf("}\\n"); return 0;}\n'
    b = probe(src2, "g++", ["-std=c++17"])
    res = {**a, **b, "source": "include/sylver/sylver.h:19-71, src/sylver_ciface.hxx:39-87",
           "generated_by": "tests/golden/make_layouts.py (gcc/g++, LP64)"}
    json.dump(res, open(OUT, "w"), indent=1)
    print(json.dumps(res, indent=1))


if __name__ == "__main__":
    sys.exit(main())
