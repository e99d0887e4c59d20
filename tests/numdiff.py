"""Numeric text comparison in the spirit of numdiff, which the reference's
CI uses on res.data and stdout (.github/workflows/ci.yml:178-203): the two
texts must have the same tokens, non-numeric tokens equal, numeric tokens
within an absolute or relative tolerance (NaN equals NaN)."""
import math
import re

_NUM = re.compile(r"^[+-]?(\d+\.?\d*|\.\d+)([eE][+-]?\d+)?$|^[+-]?(NaN|inf)$")


def tokens(text):
    return re.split(r"[\s|:]+", text.strip())


def compare(a, b, abs_tol=0.0, rel_tol=0.0):
    """Returns a list of (index, token_a, token_b) differences."""
    ta, tb = tokens(a), tokens(b)
    if len(ta) != len(tb):
        return [(-1, len(ta), len(tb))]
    bad = []
    for i, (x, y) in enumerate(zip(ta, tb)):
        if x == y:
            continue
        if _NUM.match(x) and _NUM.match(y):
            fx, fy = float(x), float(y)
            if math.isnan(fx) and math.isnan(fy):
                continue
            d = abs(fx - fy)
            if d <= abs_tol or d <= rel_tol * max(abs(fx), abs(fy)):
                continue
        bad.append((i, x, y))
    return bad
