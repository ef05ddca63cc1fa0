"""The engine's built-in size-class table (kDefaultTuning in
csrc/r2p_engine.cu) is the autotuner's committed GB300 result
(tuning_gb300.json): the two must not drift apart."""
import json
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "raw2png-conversionthrugpu_gb300")


def builtin_table():
    src = open(os.path.join(PKG, "csrc", "r2p_engine.cu")).read()
    body = re.search(r"kDefaultTuning\s*=\s*\{(.*?)\};", src, re.S).group(1)
    rows = []
    for m in re.finditer(r"\{\s*([^{}]+?)\s*\}", body):
        f = [x.strip() for x in m.group(1).split(",")]
        rows.append([2 ** 62 if f[0] == "~0ull" else int(f[0].rstrip("ull")), int(f[1]), int(f[2]), int(f[3])])
    return rows


def test_builtin_table_is_the_autotuned_one():
    tuned = json.load(open(os.path.join(PKG, "tuning_gb300.json")))["classes"]
    assert tuned[-1][0] >= 2 ** 62
    assert builtin_table() == [[min(c[0], 2 ** 62)] + c[1:] for c in tuned]
