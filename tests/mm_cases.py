"""Matrix Market texts for the reader tests: value spellings strtod accepts
(signs, missing integer or fraction digits, exponents, more than 19 digits,
ties of the round-to-nearest-even rule, values outside the device's exact
path), separators, CRLF line ends, duplicates and mirrored entries."""
import numpy as np

# (text, how it must read): ties, boundaries of the exact path, host-path forms
SPECIAL_VALUES = [
    "0", "-0", "+0.0", "-0.000", "1", "-1", "+2.5", ".5", "5.", "-.25e1", "1e0", "1E+00",
    "3.25E+02", "1e-5", "-7.0000000000000000e-01", "0.1", "0.2", "0.3",
    "9007199254740993",        # 2^53 + 1: tie, rounds to the even 2^53
    "9007199254740995",        # tie, rounds up to 2^53 + 4
    "9007199254740994",        # exact
    "18014398509481985",       # 2^54 + 1: below the tie, rounds down
    "1234567890123456789",     # 19 digits
    "9999999999999999999",     # 19 nines
    "12345678901234567890",    # 20 digits: the host parses it
    "0.12345678901234567890123",  # 23 digits: the host
    "1e27", "1e-27", "9.99e26", "123456789e-27", "1e28", "1e-28", "1e300", "1e-300",
    "4.9406564584124654e-324", "2.2250738585072014e-308", "1.7976931348623157e308",
    "0.000000000000000000000000000123",  # leading zeros do not count as digits
    "1.50000000000000000000",            # trailing zeros past 19 digits: the host
    "7.0e-3", "-6.02214076e23", "6.62607015e-34", "2.718281828459045",
    "3.141592653589793238", "1.0000000000000002", "0.9999999999999999",
]


def value_strings(rng, count):
    """Random spellings: repr, fixed-width exponent, %g, integers, and random
    1-19 digit mantissas with decimal exponents in [-40, 40]."""
    out = []
    for _ in range(count):
        k = rng.integers(0, 6)
        x = float(np.exp(rng.normal(0, 3))) * (1 if rng.random() < 0.7 else -1)
        if k == 0:
            out.append(repr(x))
        elif k == 1:
            out.append(f"{x:.17g}")
        elif k == 2:
            out.append(f"{x:.6e}")
        elif k == 3:
            out.append(f"{x:g}")
        elif k == 4:
            out.append(str(int(rng.integers(-10**6, 10**6))))
        else:
            nd = int(rng.integers(1, 20))
            mant = int(rng.integers(10 ** (nd - 1), 10 ** nd, dtype=np.uint64)) if nd < 19 else \
                int(rng.integers(10**18, 2**63 - 1, dtype=np.int64))
            out.append(f"{mant}e{int(rng.integers(-40, 41))}")
    return out


def general_text(seed=1, n=60, m=50, entries=600, crlf=True):
    """'coordinate real general', rows/cols at random with duplicates, every
    value spelling above, tabs and spaces as separators."""
    rng = np.random.default_rng(seed)
    vals = SPECIAL_VALUES + value_strings(rng, entries - len(SPECIAL_VALUES))
    rows = rng.integers(1, n + 1, entries)
    cols = rng.integers(1, m + 1, entries)
    dup = rng.random(entries) < 0.1  # repeat an earlier position
    for i in np.nonzero(dup)[0]:
        if i > 0:
            j = rng.integers(0, i)
            rows[i], cols[i] = rows[j], cols[j]
    lines = ["%%MatrixMarket matrix coordinate real general", "% generated", f"{n} {m} {entries}"]
    for i in range(entries):
        sep = "\t" if rng.random() < 0.2 else " " * int(rng.integers(1, 3))
        end = "\r" if crlf and rng.random() < 0.2 else (" " if rng.random() < 0.1 else "")
        lines.append(f"{rows[i]}{sep}{cols[i]}{sep}{vals[i]}{end}")
    return "\n".join(lines) + "\n"


def symmetric_text(seed=2, n=40, entries=300):
    """'coordinate real symmetric': diagonal entries, both triangles, duplicates."""
    rng = np.random.default_rng(seed)
    vals = value_strings(rng, entries)
    rows = rng.integers(1, n + 1, entries)
    cols = np.where(rng.random(entries) < 0.2, rows, rng.integers(1, n + 1, entries))
    lines = ["%%MatrixMarket matrix coordinate real symmetric", f"{n} {n} {entries}"]
    lines += [f"{rows[i]} {cols[i]} {vals[i]}" for i in range(entries)]
    return "\n".join(lines) + "\n"


def pattern_text(seed=3, n=30, entries=120):
    rng = np.random.default_rng(seed)
    rows = rng.integers(1, n + 1, entries)
    cols = rng.integers(1, n + 1, entries)
    lines = ["%%MatrixMarket matrix coordinate pattern symmetric", f"{n} {n} {entries}"]
    lines += [f"{rows[i]} {cols[i]}" for i in range(entries)]
    return "\n".join(lines)  # no newline after the last entry


def with_comments_and_blanks(text, seed=4):
    """Comment and blank lines inside the data (skipped by this library's
    readers; the reference's fgets loop would count them as entries)."""
    rng = np.random.default_rng(seed)
    lines = text.split("\n")
    head, body = lines[:3], lines[3:]
    out = list(head)
    for ln in body:
        r = rng.random()
        if r < 0.05:
            out.append("% a comment line")
        elif r < 0.1:
            out.append("   ")
        out.append(ln)
    return "\n".join(out)
