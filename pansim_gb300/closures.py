"""Closure rules on the host side of the C ABI.

Rules use the closureRules.json format of the reference
(include/IO/inputFormats/closuresFormat.h:7-22: name, conditionType,
threshold, threshold2, parameter, closeAfter, openAfter,
locationTypesToClose); `rule_array` packs them into psim_closure_rule
structs for psim_closures_init.  Numeric parameters are passed as text and
parsed by the library as the reference does (std::stod / std::stoi).
"""
import json

from . import cabi

STATS_COLUMNS = ["H", "T", "P1", "P2", "Q", "QT", "NQ", "MUT", "HOM", "VAC", "NI", "INF", "REINF", "BSTR", "IMM",
                 "HCI", "HCE", "INFV", "INFH", "VNI"]


def stats_header(state_names):
    """statesHeader of simulation.h:749: the state names, each followed by a
    tab, then the fixed columns."""
    return "".join(n + "\t" for n in state_names) + "\t".join(STATS_COLUMNS)


def _param_text(v):
    if isinstance(v, str):
        return v
    if isinstance(v, bool):
        return "1" if v else "0"
    if isinstance(v, int):
        return str(v)
    return repr(float(v))


def rule_array(rules):
    """dicts with the closureRules.json keys -> ctypes array of PsimClosureRule."""
    arr = (cabi.PsimClosureRule * max(len(rules), 1))()
    for i, r in enumerate(rules):
        s = arr[i]
        s.name = r["name"].encode()[:63]
        s.condition_type = r.get("conditionType", "").encode()[:31]
        s.threshold = float(r.get("threshold", 0.0))
        s.threshold2 = float(r.get("threshold2", 0.0))
        s.parameter = _param_text(r.get("parameter", "")).encode()[:63]
        s.close_after = int(r.get("closeAfter", 0))
        s.open_after = int(r.get("openAfter", 0))
        types = list(r.get("locationTypesToClose", []))
        if len(types) > cabi.PSIM_CLOSURE_MAX_TYPES:
            raise ValueError("rule %s lists more than %d location types" % (r["name"], cabi.PSIM_CLOSURE_MAX_TYPES))
        s.n_types = len(types)
        for j, t in enumerate(types):
            s.types[j] = int(t)
    if not rules:
        return (cabi.PsimClosureRule * 0)()
    return arr


def load_rules(path):
    """The `rules` list of a closureRules.json file."""
    with open(path) as f:
        return json.load(f)["rules"]
