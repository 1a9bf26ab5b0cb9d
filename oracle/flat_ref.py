"""Oracle of the element result files (test infrastructure only): the Fortran E15.6 edit
descriptor of oupestr's `write(fid, '(30e15.6)')` (src/ouresult.f:271-300) restated with
Python's correctly rounded decimal conversion (round half to even), and the line layout
of ouelestr (src/ouresult.f:140-262): six components then zeros, 26 values a line for
stresses (num_short_stress + 15) and 22 for strains (num_short_strain + 15), values with
|v| < 1e-30 written as zero."""


def e15_6(v):
    """Fortran E15.6: 0.dddddd E+ee, right-justified in 15 columns."""
    v = float(v)
    if v == 0.0:
        return "0.000000E+00".rjust(15)
    mant, ex = format(abs(v), ".5e").split("e")
    e = int(ex) + 1
    body = "0." + mant.replace(".", "") + ("E%+03d" % e if abs(e) <= 99 else "%+04d" % e)
    return ("-" + body if v < 0 else body).rjust(15)


def flat_text(comps, nvals):
    """comps: (6, N3) array (history words of the quantity); nvals: 26 or 22."""
    out = []
    zero = e15_6(0.0)
    for v in range(comps.shape[1]):
        fields = []
        for j in range(6):
            x = float(comps[j, v])
            if abs(x) < 1.0e-30:
                x = 0.0
            fields.append(e15_6(x))
        fields += [zero] * (nvals - 6)
        out.append("".join(fields) + "\n")
    return "".join(out)
