"""Writes case_tables.inc: the Unicode case mappings and alphabetic ranges
that UPPER / LOWER / INITCAP use on the device, from the Unicode Character
Database as Python's unicodedata holds it.

Per code point: its uppercase and lowercase mapping (one code point, or up to
three for the unconditional SpecialCasing entries such as U+00DF -> "SS"),
and whether it is alphabetic (general category L*), which delimits INITCAP's
words.  Run it with the interpreter whose Unicode version the oracle uses:
    python gen_case_tables.py > case_tables.inc
"""
import sys
import unicodedata


def main(out=sys.stdout):
    up1, lo1, upm, lom, alpha = [], [], [], [], []
    start = None
    for cp in range(0x110000):
        if 0xD800 <= cp <= 0xDFFF:
            a = False
        else:
            c = chr(cp)
            u, l = c.upper(), c.lower()
            if u != c:
                (up1 if len(u) == 1 else upm).append((cp, [ord(x) for x in u]))
            if l != c:
                (lo1 if len(l) == 1 else lom).append((cp, [ord(x) for x in l]))
            a = c.isalpha()
        if a and start is None:
            start = cp
        if not a and start is not None:
            alpha.append((start, cp - 1))
            start = None
    w = out.write
    w("// Generated by gen_case_tables.py from the Unicode Character Database %s\n" % unicodedata.unidata_version)
    w("// (Python %d.%d unicodedata).  Do not edit.\n" % sys.version_info[:2])
    w('#define GX_CASE_UNICODE_VERSION "%s"\n' % unicodedata.unidata_version)

    def arr(name, vals, per=12):
        w("__device__ const uint32_t %s[%d] = {\n" % (name, len(vals)))
        for i in range(0, len(vals), per):
            w("    " + ", ".join("0x%x" % v for v in vals[i:i + per]) + ",\n")
        w("};\n")
    for name, pairs in (("kUpper", up1), ("kLower", lo1)):
        w("constexpr int %sCount = %d;\n" % (name, len(pairs)))
        arr(name + "From", [p[0] for p in pairs])
        arr(name + "To", [p[1][0] for p in pairs])
    for name, pairs in (("kUpperMulti", upm), ("kLowerMulti", lom)):
        assert all(len(p[1]) <= 3 for p in pairs)
        w("constexpr int %sCount = %d;\n" % (name, len(pairs)))
        arr(name + "From", [p[0] for p in pairs])
        arr(name + "To", [x for p in pairs for x in (p[1] + [0, 0, 0])[:3]])
    w("constexpr int kAlphaCount = %d;\n" % len(alpha))
    arr("kAlphaLo", [a[0] for a in alpha])
    arr("kAlphaHi", [a[1] for a in alpha])


if __name__ == "__main__":
    main()
