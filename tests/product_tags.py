"""Parse reference tag reprs into carcassonne_gb300.sparse tag objects."""
import re

from carcassonne_gb300.sparse import Complete, Identity, OneSiteOperator, TwoSiteOperator, TwoSiteOperatorCompressed


def parse(s):
    s = s.strip()
    if s == "Identity()":
        return Identity()
    if s == "Complete()":
        return Complete()
    if s.startswith("OneSiteOperator("):
        return OneSiteOperator(None)
    m = re.fullmatch(r"TwoSiteOperator\((\d+),(\d+),(None|-?\d+)\)", s)
    if m:
        return TwoSiteOperator(int(m.group(1)), int(m.group(2)), None if m.group(3) == "None" else int(m.group(3)))
    m = re.fullmatch(r"TwoSiteOperatorCompressed\((\d+)\)", s)
    if m:
        return TwoSiteOperatorCompressed(int(m.group(1)))
    raise ValueError(s)
