"""Generate ``clblm_ref_tables.h``: the numeric tables CLBLM's line-by-line
path reads from its Fortran source.

The tables must be identical to the reference's for the results to be
identical, so they are extracted from the reference source text rather than
retyped.  The decimal literals are carried over verbatim; both gfortran
(``-fdefault-real-8``) and a C compiler parse such a literal straight to the
nearest binary64 value, so the tables are bit-identical.

Tables extracted (reference file:line):
  * Voigt-width / sub-function weights AVRAT, CGAUSS, CF1, CF2, CF3, CER
    (102 entries each over zeta = 0, 0.01, ..., 1.01):
    src/clblm_src/clblm_ODLAY_CommonSub.f90:43-185
  * TIPS temperature grid Tdat(119):  src/clblm_src/clblm_ODLAY_TIPS.f90:16-29
  * TIPS Q(T): every ``QofT(k,J)`` DATA row of the 45 QT_* routines
    (src/clblm_src/clblm_ODLAY_TIPS.f90:421-5442), and for each HITRAN
    molecule 1-47 and isotopologue the row TIPS_2003's dispatch (:57-419)
    reads: the isotopologue's own, the first isotopologue's where the
    dispatch falls back to it (HNO3, HF, HCl, HBr, HI, N2, COF2), none where
    it sets Q = 1 (O, CH3OH, SO3)
  * the number of isotopologues of each molecule (MaxISOTPL_smass) and their
    molecular masses (isotpl_mass): src/common/clblm_ConstParam.f90:246-420
  * CO2 continuum (mt_ckd 2.5): FRNCO2's coefficients S(1:5003) on -4 to
    10000 cm-1 at 2 cm-1 and its band-head temperature exponents
    TDEP_BANDHEAD(1196:1220), src/clblm_src/clblm_ODLAY_Continuum.f90:1333-2511;
    CONTNM's XFACCO2(500) scaling for 2000-2998 cm-1, :145-204
  * N2 continua: the pure-rotation band's C and SF at 296 K and 220 K
    (xn2_r, 73 points on -10..350 cm-1), the fundamental's coefficients at
    272 K and 228 K and the H2O efficiencies (n2_ver_1, 230 points from
    1993.8 cm-1), the first overtone's coefficients (n2_overtone1, 201
    points from 4325 cm-1)
  * O3 continua: Chappuis X, Y, Z (XO3CHP, 3150 points from 8920 cm-1),
    Hartley-Huggins at 0 C and its linear and quadratic temperature
    coefficients (O3HHT0/1/2, 2687 points from 27370 cm-1), the UV
    (O3HHUV, 133 points from 40800 cm-1)
  * O2 continua: the fundamental's XO2, XO2T (o2_ver_1, 103 points from
    1340 cm-1), the 1.27 um band (O2INF1, 483 from 7536), the A band
    (O2INF3, 261 from 12961.5), the visible (O2_vis, 1488 from 15000), the
    far UV (O2FUV, 1512 from 56740)

Run (in a tree where the reference is mounted):
    python clblm_gb300/csrc/gen_ref_tables.py <CLBLM source root> > clblm_gb300/csrc/clblm_ref_tables.h
The generated header is committed; the build never needs the reference.
"""
import re
import sys
from pathlib import Path

NUM = r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[EeDd][-+]?\d+)?"


def _numbers(text):
    """The values of a DATA list, a repeat count N*value expanded."""
    out = []
    for rep, tok in re.findall(r"(?:(\d+)\s*\*\s*)?(%s)" % NUM, text):
        out.extend([tok.replace("D", "E").replace("d", "e")] * (int(rep) if rep else 1))
    return out


def _fortran_array(src, name):
    m = re.search(r"real\s*,\s*PARAMETER\s*::\s*%s\s*\(1:102\)\s*=\s*\[(.*?)\]" % name,
                  src, re.S | re.I)
    if not m:
        raise SystemExit("table %s not found" % name)
    body = "\n".join(line.split("!")[0] for line in m.group(1).splitlines())
    vals = _numbers(body)
    if len(vals) != 102:
        raise SystemExit("table %s: %d values" % (name, len(vals)))
    return vals


def _tips_grid(src):
    m = re.search(r"Tdat\(NT\)\s*=\s*\[(.*?)\]", src, re.S)
    vals = _numbers(m.group(1).replace("&", " "))
    if len(vals) != 119:
        raise SystemExit("Tdat: %d values" % len(vals))
    return vals


def _tips_all(src, maxiso):
    """(rows, rowmap): the Q(T) rows of all QT_* routines in file order, and
    rowmap[mol-1][iso-1] = the row TIPS_2003 interpolates for (mol, iso);
    -1 where it takes Q = 1."""
    subs = [(m.group(1), m.start()) for m in re.finditer(r"Subroutine\s+QT_(\w+)\s*\(", src, re.I)]
    rows, first = [], {}
    for k, (name, pos) in enumerate(subs):
        body = src[pos:subs[k + 1][1] if k + 1 < len(subs) else len(src)]
        nrow = int(re.search(r"dimension\s+xgj\(\s*(\d+)\)", body, re.I).group(1))
        first[name.upper()] = (len(rows), nrow)
        for j in range(1, nrow + 1):
            m = re.search(r"data\s*\(QofT\(\s*%d\s*,\s*J\)\s*,\s*J=1,119\)\s*/(.*?)/" % j, body, re.S | re.I)
            text = "\n".join(line.split("!")[0] for line in m.group(1).splitlines())
            vals = _numbers(text.replace("&", " "))
            if len(vals) != 119:
                raise SystemExit("QT_%s row %d: %d values" % (name, j, len(vals)))
            rows.append(vals)
    disp = src[src.index("Subroutine TIPS_2003"):subs[0][1]]
    rowmap = []
    for mol in range(1, 48):
        blk = re.search(r"IF\s*\(\s*MOL\s*\.EQ\.\s*%d\s*\)\s*THEN(.*?)go to 100" % mol, disp, re.I | re.S)
        call = re.search(r"CALL\s+QT_(\w+)\s*\(", blk.group(1), re.I)
        if not call:
            if not re.search(r"QT\s*=\s*1", blk.group(1), re.I):
                raise SystemExit("molecule %d: no TIPS routine and no Q = 1" % mol)
            rowmap.append([-1] * maxiso[mol - 1])
            continue
        base, nrow = first[call.group(1).upper()]
        own = nrow
        g = re.search(r"IF\s*\(\s*ISO\.EQ\.1\s*(\.OR\.\s*ISO\s*\.EQ\.\s*2)?\s*\)", blk.group(1), re.I)
        if g:
            own = 2 if g.group(1) else 1
        elif maxiso[mol - 1] > nrow:
            raise SystemExit("molecule %d: %d isotopologues, %d TIPS rows" % (mol, maxiso[mol - 1], nrow))
        rowmap.append([base + (iso - 1 if iso <= own else 0) for iso in range(1, maxiso[mol - 1] + 1)])
    return rows, rowmap


def _maxiso(src):
    m = re.search(r"MaxISOTPL_smass\(MXMOL\)\s*=\s*\[(.*?)\]", src, re.S)
    text = "\n".join(line.split("!")[0] for line in m.group(1).splitlines())
    vals = [int(v) for v in re.findall(r"\d+", text.replace("&", " "))]
    if len(vals) != 47:
        raise SystemExit("MaxISOTPL_smass: %d values" % len(vals))
    return vals


def _masses_all(src, maxiso):
    out = []
    for m_id in range(1, 48):
        m = re.search(r"data\s*\(isotpl_mass\(%d,i\),i=1,(\d+)\)\s*&?\s*&?\s*/(.*?)/" % m_id, src, re.S | re.I)
        if not m:
            raise SystemExit("masses of molecule %d not found" % m_id)
        text = "\n".join(line.split("!")[0] for line in m.group(2).splitlines())
        vals = _numbers(text.replace("&", " "))
        if len(vals) != int(m.group(1)) or len(vals) < maxiso[m_id - 1]:
            raise SystemExit("masses of molecule %d: %d values" % (m_id, len(vals)))
        out.append(vals[:maxiso[m_id - 1]])
    return out


def _data_block(src, start_pat, data_pat, count):
    """The values of a DATA statement (after start_pat) with `count` entries."""
    st = re.search(start_pat, src, re.I)
    if not st:
        raise SystemExit("%s not found" % start_pat)
    # comments first: they hold slashes of their own (the "!DATA F0000/" labels)
    text = "\n".join(line.split("!")[0] for line in src[st.start():].splitlines())
    m = re.search(data_pat, text, re.S | re.I)
    if not m:
        raise SystemExit("%s: data not found" % data_pat)
    vals = _numbers(m.group(1).replace("&", " "))
    if len(vals) != count:
        raise SystemExit("%s: %d values, want %d" % (data_pat, len(vals), count))
    return vals


def _data_segments(src, start_pat, name, count):
    """An array filled by segments DATA (NAME(I),I= a, b)/.../ after start_pat."""
    st = re.search(start_pat, src, re.I)
    if not st:
        raise SystemExit("%s not found" % start_pat)
    end = re.search(r"END\s+SUBROUTINE", src[st.end():], re.I)
    text = "\n".join(line.split("!")[0] for line in src[st.start():st.end() + end.start()].splitlines())
    vals = [None] * count
    for m in re.finditer(r"DATA\s*\(\s*%s\s*\(\s*I\s*\)\s*,\s*I\s*=\s*(\d+)\s*,\s*(\d+)\s*\)\s*/(.*?)/" % name,
                         text, re.S | re.I):
        a, b = int(m.group(1)), int(m.group(2))
        seg = _numbers(m.group(3).replace("&", " "))
        if len(seg) != b - a + 1:
            raise SystemExit("%s(%d:%d): %d values" % (name, a, b, len(seg)))
        vals[a - 1:b] = seg
    if any(v is None for v in vals):
        raise SystemExit("%s: %d of %d values" % (name, sum(v is not None for v in vals), count))
    return vals


def main(ref_root):
    ref = Path(ref_root)
    common = (ref / "src/clblm_src/clblm_ODLAY_CommonSub.f90").read_text(errors="replace")
    tips = (ref / "src/clblm_src/clblm_ODLAY_TIPS.f90").read_text(errors="replace")
    const = (ref / "src/common/clblm_ConstParam.f90").read_text(errors="replace")

    lines = [
        "/* Generated by gen_ref_tables.py from the CLBLM Fortran source; do not edit.",
        " * Decimal literals are carried over verbatim so that the binary64 values match",
        " * the reference's (-fdefault-real-8) tables bit for bit. */",
        "#ifndef CLBLM_REF_TABLES_H",
        "#define CLBLM_REF_TABLES_H",
        "",
    ]

    def emit(name, vals, per=5):
        lines.append("static const double %s[%d] = {" % (name, len(vals)))
        for i in range(0, len(vals), per):
            lines.append("    " + ", ".join(vals[i:i + per]) + ",")
        lines.append("};")
        lines.append("")

    # clblm_ODLAY_CommonSub.f90:43-185
    for name in ("AVRAT", "CGAUSS", "CF1", "CF2", "CF3", "CER"):
        emit("CLBLM_" + name, _fortran_array(common, name))
    # clblm_ODLAY_TIPS.f90:16-29
    emit("CLBLM_TIPS_TDAT", _tips_grid(tips), per=8)
    # MaxISOTPL_smass and isotpl_mass, clblm_ConstParam.f90:246-420
    maxiso = _maxiso(const)
    lines.append("#define CLBLM_MXMOL 47   /* MXMOL */")
    lines.append("#define CLBLM_MXISO 10   /* isotopologues of a molecule at most */")
    lines.append("static const int CLBLM_MAXISO[47] = {")
    lines.append("    " + ", ".join(str(v) for v in maxiso) + ",")
    lines.append("};")
    lines.append("")
    lines.append("/* molecular mass of (molecule, isotopologue); 0: no such isotopologue */")
    lines.append("static const double CLBLM_ISO_MASS[47][10] = {")
    for vals in _masses_all(const, maxiso):
        lines.append("    {" + ", ".join(vals + ["0."] * (10 - len(vals))) + "},")
    lines.append("};")
    lines.append("")
    rows, rowmap = _tips_all(tips, maxiso)
    lines.append("/* TIPS Q(T) rows of the QT_* routines, in file order */")
    lines.append("#define CLBLM_TIPS_NQ %d" % len(rows))
    lines.append("static const double CLBLM_TIPS_Q[%d][119] = {" % len(rows))
    for vals in rows:
        lines.append("  {")
        for i in range(0, len(vals), 6):
            lines.append("    " + ", ".join(vals[i:i + 6]) + ",")
        lines.append("  },")
    lines.append("};")
    lines.append("")
    lines.append("/* the row of CLBLM_TIPS_Q for (molecule, isotopologue); -1: Q = 1; -2: no such isotopologue */")
    lines.append("static const int CLBLM_TIPS_QROW[47][10] = {")
    for r in rowmap:
        lines.append("    {" + ", ".join(str(v) for v in r + [-2] * (10 - len(r))) + "},")
    lines.append("};")
    lines.append("")
    # clblm_ODLAY_Continuum.f90: FRNCO2 (:1333-2511) and CONTNM's XFACCO2 (:145-204)
    cont = (ref / "src/clblm_src/clblm_ODLAY_Continuum.f90").read_text(errors="replace")
    emit("CLBLM_CO2_S", _data_block(cont, r"SUBROUTINE\s+FRNCO2", r"DATA\s+S\(1:5003\)\s*/(.*?)/", 5003))
    emit("CLBLM_CO2_TDEP", _data_block(cont, r"SUBROUTINE\s+FRNCO2",
                                       r"data\s*\(tdep_bandhead\(i\),i=1196,1220\)\s*/(.*?)/", 25))
    emit("CLBLM_XFACCO2", _data_block(cont, r"SUBROUTINE\s+CONTNM", r"DATA\s+XFACCO2\s*/(.*?)/", 500), per=8)
    # N2 continua: xn2_r (:2533-2681), n2_ver_1 (:2696-2945), n2_overtone1 (:2948-3056)
    for name, pat in (("C_296", r"DATA\s+C_296\(1:73\)\s*/(.*?)/"), ("SF_296", r"DATA\s+sf_296\s*/(.*?)/"),
                      ("C_220", r"DATA\s+C_220\(1:73\)\s*/(.*?)/"), ("SF_220", r"DATA\s+sf_220\s*/(.*?)/")):
        emit("CLBLM_N2R_" + name, _data_block(cont, r"SUBROUTINE\s+xn2_r", pat, 73))
    for name in ("xn2_272", "xn2_228", "a_h2o"):
        emit("CLBLM_N2F_" + name.upper(),
             _data_block(cont, r"subroutine\s+n2_ver_1", r"DATA\s+%s\s*/(.*?)/" % name, 230))
    emit("CLBLM_N2O1_XN2", _data_block(cont, r"subroutine\s+n2_overtone1", r"DATA\s+xn2\s*/(.*?)/", 201))
    # O3 continua: XO3CHP (:3061-5205), O3HHT0/1/2 (:5210-7085), O3HHUV (:7090-7175)
    for name in ("X", "Y", "Z"):
        emit("CLBLM_O3CHP_" + name, _data_segments(cont, r"SUBROUTINE\s+XO3CHP", name, 3150))
    for sub in ("O3HHT0", "O3HHT1", "O3HHT2"):
        emit("CLBLM_" + sub, _data_block(cont, r"SUBROUTINE\s+%s\b" % sub, r"DATA\s+S\(1:2687\)\s*/(.*?)/", 2687))
    emit("CLBLM_O3HHUV", _data_block(cont, r"SUBROUTINE\s+O3HHUV", r"DATA\s+S\(1:133\)\s*/(.*?)/", 133))
    # O2 continua: o2_ver_1 (:7180-7310), O2INF1 (:7327-7488), O2INF3 (:7573-7682),
    # O2_vis (:7699-8090), O2FUV (:8257-8770)
    emit("CLBLM_O2F_XO2", _data_block(cont, r"subroutine\s+o2_ver_1", r"DATA\s+xo2\(1:103\)\s*/(.*?)/", 103))
    emit("CLBLM_O2F_XO2T", _data_block(cont, r"subroutine\s+o2_ver_1", r"DATA\s+xo2t\(1:103\)\s*/(.*?)/", 103))
    emit("CLBLM_O2INF1", _data_block(cont, r"SUBROUTINE\s+O2INF1", r"DATA\s+xo2inf1\(1:483\)\s*/(.*?)/", 483))
    emit("CLBLM_O2INF3", _data_block(cont, r"SUBROUTINE\s+O2INF3", r"DATA\s+xo2inf3\s*/(.*?)/", 261))
    emit("CLBLM_O2VIS", _data_block(cont, r"SUBROUTINE\s+O2_vis", r"DATA\s+S\(1:1488\)\s*/(.*?)/", 1488))
    emit("CLBLM_O2FUV", _data_block(cont, r"SUBROUTINE\s+O2FUV", r"DATA\s+S\(1:1512\)\s*/(.*?)/", 1512))
    lines.append("#endif")
    sys.stdout.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: gen_ref_tables.py <CLBLM source root>  (the directory holding src/)")
    main(sys.argv[1])
