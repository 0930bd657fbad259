"""The libgbpa drop-in as edits of MFEM's fem/bilinearform_ext.cpp.

Three hooks, each inserted at an anchor that must occur exactly once in the
source (otherwise the patch refuses, naming the anchor):
  - the shim's header after the file's own includes;
  - gbpa_shim::Assemble at the end of PABilinearFormExtension::Assemble;
  - gbpa_shim::Mult at the start of PABilinearFormExtension::MultInternal
    (y = A x through libgbpa when the form is forwarded);
  - gbpa_shim::Release at the start of PABilinearFormExtension::Update.
No class layout changes, so every other object of an existing MFEM build is
reused as is. mfem_gbpa.patch is the same change as a unified diff (for
`git apply` / `patch -p1` inside an MFEM tree); this script is what the build
uses, because it needs neither tool.

    python3 mfem_gbpa_patch.py <MFEM source tree> <output tree>
        writes <output tree>/fem/bilinearform_ext.cpp
    python3 mfem_gbpa_patch.py --diff <MFEM source tree>
        prints the unified diff (the content of mfem_gbpa.patch)
"""
import difflib
import os
import sys

FILE = os.path.join("fem", "bilinearform_ext.cpp")

EDITS = [
    ('#include "ceed/interface/util.hpp"\n',
     '#include "ceed/interface/util.hpp"\n#include "gbpa_shim.hpp"\n'),
    ("      integ->AssemblePABoundaryFaces(*a->FESpace());\n   }\n}\n",
     "      integ->AssemblePABoundaryFaces(*a->FESpace());\n   }\n\n"
     "   // libgbpa: the form's operator from the arrays assembled above\n"
     "   gbpa_shim::Assemble(this, *a, elem_restrict);\n}\n"),
    ("void PABilinearFormExtension::Update()\n{\n",
     "void PABilinearFormExtension::Update()\n{\n   gbpa_shim::Release(this);\n"),
    ("void PABilinearFormExtension::MultInternal(const Vector &x, Vector &y,\n"
     "                                           const bool useAbs) const\n{\n",
     "void PABilinearFormExtension::MultInternal(const Vector &x, Vector &y,\n"
     "                                           const bool useAbs) const\n{\n"
     "   // libgbpa: restriction, apply and transpose on the GPU\n"
     "   if (!useAbs && gbpa_shim::Mult(this, *a, x, y)) { return; }\n\n"),
]


def patched(src):
    out = src
    for anchor, repl in EDITS:
        n = out.count(anchor)
        if n != 1:
            raise SystemExit(f"{FILE}: anchor found {n} times, expected once:\n{anchor}")
        out = out.replace(anchor, repl)
    return out


def diff(ref):
    with open(os.path.join(ref, FILE)) as f:
        src = f.read()
    lines = difflib.unified_diff(src.splitlines(True), patched(src).splitlines(True),
                                 "a/" + FILE.replace(os.sep, "/"), "b/" + FILE.replace(os.sep, "/"))
    return "".join(lines)


def main():
    if len(sys.argv) == 3 and sys.argv[1] == "--diff":
        sys.stdout.write(diff(sys.argv[2]))
        return
    if len(sys.argv) != 3:
        raise SystemExit(__doc__)
    ref, out = sys.argv[1], sys.argv[2]
    with open(os.path.join(ref, FILE)) as f:
        src = f.read()
    dst = os.path.join(out, FILE)
    os.makedirs(os.path.dirname(dst), exist_ok=True)
    with open(dst, "w") as f:
        f.write(patched(src))


if __name__ == "__main__":
    main()
