"""Conversion between the reference's tag reprs and the oracle's tuple tags."""
import re


def parse_tag(s):
    s = s.strip()
    if s == "Identity()":
        return ("I",)
    if s == "Complete()":
        return ("C",)
    m = re.fullmatch(r"OneSiteOperator\((.*)\)", s)
    if m:
        return ("O", None)
    m = re.fullmatch(r"TwoSiteOperator\((\d+),(\d+),(None|-?\d+)\)", s)
    if m:
        pos = None if m.group(3) == "None" else int(m.group(3))
        return ("T", int(m.group(1)), int(m.group(2)), pos)
    m = re.fullmatch(r"TwoSiteOperatorCompressed\((\d+)\)", s)
    if m:
        return ("TC", int(m.group(1)))
    raise ValueError(s)


def tag_repr(t):
    if t[0] == "I":
        return "Identity()"
    if t[0] == "C":
        return "Complete()"
    if t[0] == "O":
        return "OneSiteOperator(None)"
    if t[0] == "T":
        return "TwoSiteOperator({},{},{})".format(t[1], t[2], t[3])
    return "TwoSiteOperatorCompressed({})".format(t[1])
