"""Recipe that extracts the physical data tables (no algorithm code) used by the
oracle and by the GPU library from the reference checkout.

The tables are measured/evaluated physical data that both implementations must
hold identically: Geant4 atomic-shell occupancies and binding energies (used by
the Fano density effect of the electronic stopping power), nuclear RMS radii
(polar angle of radiative hard events, Coulomb nuclear form factor) and the
Salvat (1987) screening amplitudes/exponents (Coulomb tables).  Everything
else (quadrature nodes, dilogarithm, models) is computed by our own code.

Sources (reference project paths):
  src/Materials.jl        _ATOMIC_SHELL_INDEX
  src/AtomicShellData.jl  _ATOMIC_SHELL_OCCUPANCY, _ATOMIC_SHELL_ENERGY
  src/Straggling.jl       NUCLEAR_RMS_RADII
  src/Coulomb.jl          SALVAT_PREFACTOR, SALVAT_EXPONENT, NUCLEAR_RADII

Usage: python oracle/gen_physics_data.py <path of the reference checkout>
Writes oracle/physics_data.inc and diffpumas.jl_gb300/csrc/physics_data.inc
(two copies: the oracle never includes product files and vice versa).
"""
import os
import re
import sys

NUM = re.compile(r"[-+]?\d+\.?\d*(?:[eE][-+]?\d+)?")


def block(text, name):
    i = text.index("const " + name)
    j = text.index("=", i) + 1
    opener = None
    for k in range(j, len(text)):
        if text[k] in "([":
            opener = k
            break
    depth = 0
    for k in range(opener, len(text)):
        c = text[k]
        if c in "([":
            depth += 1
        elif c in ")]":
            depth -= 1
            if depth == 0:
                return text[opener:k + 1]
    raise ValueError(name)


def strip_comments(s):
    return "\n".join(line.split("#", 1)[0] for line in s.splitlines())


def flat(s):
    s = strip_comments(s)
    s = re.sub(r"\b(UInt8|UInt16|Float32|Float64)\b", "", s)
    return [float(x) for x in NUM.findall(s)]


def groups(s):
    s = strip_comments(s)
    inner = s.strip()[1:-1]
    out, depth, cur = [], 0, ""
    for c in inner:
        if c == "(":
            depth += 1
            if depth == 1:
                cur = ""
                continue
        if c == ")":
            depth -= 1
            if depth == 0:
                out.append([float(x) for x in NUM.findall(cur)])
                continue
        if depth >= 1:
            cur += c
    return out


def carr(ctype, name, vals, fmt):
    lines = []
    for i in range(0, len(vals), 8):
        lines.append("  " + ", ".join(fmt(v) for v in vals[i:i + 8]) + ",")
    return f"static const {ctype} {name}[{len(vals)}] = {{\n" + "\n".join(lines) + "\n};\n"


def main(ref):
    mat = open(os.path.join(ref, "src/Materials.jl")).read()
    shells = open(os.path.join(ref, "src/AtomicShellData.jl")).read()
    strag = open(os.path.join(ref, "src/Straggling.jl")).read()
    coul = open(os.path.join(ref, "src/Coulomb.jl")).read()
    index = [int(v) for v in flat(block(mat, "_ATOMIC_SHELL_INDEX"))]
    occ = [int(v) for v in flat(block(shells, "_ATOMIC_SHELL_OCCUPANCY"))]
    eng = flat(block(shells, "_ATOMIC_SHELL_ENERGY"))
    rms = flat(block(strag, "NUCLEAR_RMS_RADII"))
    pre = groups(block(coul, "SALVAT_PREFACTOR"))
    exp_ = groups(block(coul, "SALVAT_EXPONENT"))
    rad = flat(block(coul, "NUCLEAR_RADII"))
    assert len(index) == 101 and len(occ) == len(eng) == index[-1]
    assert len(pre) == 2 and len(exp_) == 3
    out = ["/* Physical data tables (Geant4 atomic shells, nuclear radii, Salvat 1987",
           "   screening).  Generated by oracle/gen_physics_data.py; data only. */",
           "#pragma once"]
    out.append(carr("unsigned short", "DPDATA_SHELL_INDEX", index, lambda v: str(v)))
    out.append(carr("unsigned char", "DPDATA_SHELL_OCCUPANCY", occ, lambda v: str(v)))
    # Float32 in the source: keep the float literal so both sides round identically.
    out.append(carr("float", "DPDATA_SHELL_ENERGY_EV", eng, lambda v: repr(v) + "f"))
    out.append(carr("double", "DPDATA_NUCLEAR_RMS_RADII_FM", rms, repr))
    for i, g in enumerate(pre):
        out.append(carr("double", f"DPDATA_SALVAT_PREFACTOR{i}", g, repr))
    for i, g in enumerate(exp_):
        out.append(carr("double", f"DPDATA_SALVAT_EXPONENT{i}", g, repr))
    out.append(carr("double", "DPDATA_NUCLEAR_RADII_FM", rad, repr))
    text = "\n".join(out)
    here = os.path.dirname(os.path.abspath(__file__))
    for dst in (os.path.join(here, "physics_data.inc"),
                os.path.join(here, "..", "diffpumas.jl_gb300", "csrc", "physics_data.inc")):
        with open(dst, "w") as f:
            f.write(text)
    print("shells", len(occ), "rms", len(rms), "salvat", [len(g) for g in pre], [len(g) for g in exp_], "radii", len(rad))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <path of the reference checkout>")
    main(sys.argv[1])
