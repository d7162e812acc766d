"""Write the diagram-table headers include/constants_*.h from the library's tables.

Reference-side code includes ``constants_rho.h`` and its siblings (the
reference's include/constants_*.h, generated there by devTools/comb_*.cpp) to
get the spin-index / coefficient arrays of every diagram.  These headers are
rendered from the tables libctr.so generates from the gamma matrices
(ctr_table_*), with the same array names, element types, shapes and value
formatting (``%d`` for indices, ``%+3.2f`` for coefficients, signed zeros
kept), so that such code compiles and reads the same numbers.

    python -m contractions_code_scattering_gb300.constants_headers [--out DIR]

Only the host side of libctr.so is used (no GPU needed).
"""

import argparse
import os

import numpy as np

HEADERS = {
    "constants_rho.h": ["spinIndices_rho", "lp_rp_rho", "coef_rho"],
    "constants_rhopi.h": ["spinIndices_rhopi", "ip_rhopi", "coef_rhopi"],
    "constants_pipi.h": ["spinIndices_pipi_square", "coef_pipi_square", "spinIndices_pipi_doubleTriangle",
                         "coef_pipi_doubleTriangle", "spinIndices_pipi_doubleTriangle_hor",
                         "coef_pipi_doubleTriangle_hor"],
    "constants_sigma.h": ["spinIndices_sigma", "lp_rp_sigma", "coef_sigma"],
    "constants_sigmapi.h": ["spinIndices_sigmapi_hor_fish", "coef_sigmapi_hor_fish", "spinIndices_sigmapi_triangle",
                            "ip_sigmapi_triangle", "coef_sigmapi_triangle"],
}

_NOTE = ("/* Generated by contractions_code_scattering_gb300/constants_headers.py from the\n"
         " * diagram tables libctr.so builds from the gamma matrices (ctr_table_*).\n"
         " * Do not edit.  %s */\n")


def _tokens(a):
    a = np.asarray(a)
    if a.dtype.kind == "f":
        return ["%+3.2f" % float(v) for v in a.astype(np.float64).reshape(-1)]
    return ["%d" % int(v) for v in a.reshape(-1)]


def _array(name, a):
    a = np.asarray(a)
    ctype = "float" if a.dtype.kind == "f" else "short int"
    dims = "".join("[%d]" % d for d in a.shape)
    return "static %s %s%s = { %s};\n" % (ctype, name, dims, ",".join(_tokens(a)))


def render(tables):
    """{file name: text} for the five table headers and constants.h."""
    out = {}
    for fname, names in HEADERS.items():
        guard = "CTR_" + fname.replace(".", "_").upper()
        body = "\n".join(_array(n, tables[n]) for n in names)
        out[fname] = (_NOTE % ("Arrays: " + ", ".join(names) + ".") + "#ifndef %s\n#define %s\n\n%s\n#endif\n"
                      % (guard, guard, body))
    inc = "".join("#include <%s>\n" % f for f in HEADERS)
    out["constants.h"] = (_NOTE % "Every diagram table." + "#ifndef CTR_CONSTANTS_H\n#define CTR_CONSTANTS_H\n\n"
                          + inc + "\n#endif\n")
    return out


def library_tables():
    from . import api
    return api.tables()


def write(out_dir):
    files = render(library_tables())
    for fname, text in files.items():
        with open(os.path.join(out_dir, fname), "w") as fh:
            fh.write(text)
    return sorted(files)


def main():
    here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(here, "include"))
    args = ap.parse_args()
    for f in write(args.out):
        print(os.path.join(args.out, f))


if __name__ == "__main__":
    main()
