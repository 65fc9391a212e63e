"""Emit solid_harmonics.cuh: real regular solid harmonics S_lm(x, y, z) for l <= 6
and their gradients, as straight-line device code.

S_lm is r^l Y_lm scaled by sqrt(4 pi / (2l+1)) (the convention of
jqmc/atomic_orbital.py:2353-2585), i.e. the Racah-normalised real solid
harmonics C_l^m (m >= 0) and S_l^|m| (m < 0):

    Pi_l^m(z, r^2) = sqrt((l-m)!/(l+m)!) sum_k (-1)^k 2^-l C(l,k) C(2l-2k,l) (l-2k)!/(l-2k-m)! r^2k z^(l-2k-m)
    C_l^m = sqrt(2) Pi_l^m Re (x+iy)^m,  S_l^m = sqrt(2) Pi_l^m Im (x+iy)^m,  C_l^0 = Pi_l^0.

Each harmonic is expanded to monomials x^a y^b z^c with sympy and written out
with common-subexpression elimination.  Run:  python gen_solid_harmonics.py
"""

import os
import re

import sympy as sp

x, y, z = sp.symbols("x y z", real=True)
LMAX = 6


def solid(l, m):
    r2 = x * x + y * y + z * z
    am = abs(m)
    pi_lm = 0
    for k in range((l - am) // 2 + 1):
        pi_lm += ((-1) ** k * sp.Rational(1, 2**l) * sp.binomial(l, k) * sp.binomial(2 * l - 2 * k, l)
                  * sp.factorial(l - 2 * k) / sp.factorial(l - 2 * k - am) * r2**k * z ** (l - 2 * k - am))
    pi_lm *= sp.sqrt(sp.factorial(l - am) / sp.factorial(l + am))
    if m == 0:
        return sp.expand(pi_lm)
    w = sp.expand((x + sp.I * y) ** am)
    part = sp.re(w) if m > 0 else sp.im(w)
    return sp.expand(sp.sqrt(2) * pi_lm * part)


def emit_function(l, with_grad):
    exprs = []
    for m in range(-l, l + 1):
        s = solid(l, m)
        exprs.append(s)
        if with_grad:
            exprs += [sp.diff(s, x), sp.diff(s, y), sp.diff(s, z)]
    repl, reduced = sp.cse([sp.N(e, 20) for e in exprs], symbols=sp.numbered_symbols("t"))
    lines = []
    for sym, val in repl:
        lines.append(f"  const T {sym} = {sp.ccode(val)};")
    k = 0
    for m in range(-l, l + 1):
        j = m + l
        lines.append(f"  S[{j}] = {sp.ccode(reduced[k])};")
        k += 1
        if with_grad:
            for c in range(3):
                lines.append(f"  G[{3 * j + c}] = {sp.ccode(reduced[k])};")
                k += 1
    sig = "S, T* __restrict__ G" if with_grad else "S"
    name = f"sh{'g' if with_grad else ''}_l{l}"
    body = "\n".join(lines).replace("pow(", "jq_pow(")
    # typed literals, so a float instantiation stays in float arithmetic
    body = re.sub(r"(?<![\w.])(\d+\.\d*(?:[eE][-+]?\d+)?)", r"T(\1)", body)
    return f"template <class T>\n__device__ __forceinline__ void {name}(T x, T y, T z, T* __restrict__ {sig}) {{\n{body}\n}}\n"


def main():
    out = ["// Generated by gen_solid_harmonics.py -- do not edit.",
           "// Real regular solid harmonics S_lm (Racah normalisation, index m + l) for l <= 6,",
           "// values (sh_l*) and values + gradients (shg_l*, G[3*(m+l) + xyz]).",
           "#pragma once",
           "template <class T> __device__ __forceinline__ T jq_pow(T b, int e) { T r = T(1); for (int i = 0; i < e; ++i) r *= b; return r; }",
           ""]
    for l in range(LMAX + 1):
        out.append(emit_function(l, False))
        out.append(emit_function(l, True))
    out.append("template <class T>\n__device__ __forceinline__ void solid_harmonics(int l, T x, T y, T z, T* S) {\n  switch (l) {")
    for l in range(LMAX + 1):
        out.append(f"    case {l}: sh_l{l}(x, y, z, S); break;")
    out.append("    default: break;\n  }\n}\n")
    out.append("template <class T>\n__device__ __forceinline__ void solid_harmonics_grad(int l, T x, T y, T z, T* S, T* G) {\n  switch (l) {")
    for l in range(LMAX + 1):
        out.append(f"    case {l}: shg_l{l}(x, y, z, S, G); break;")
    out.append("    default: break;\n  }\n}\n")
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "solid_harmonics.cuh")
    with open(path, "w") as f:
        f.write("\n".join(out))
    print("wrote", path)


if __name__ == "__main__":
    main()
