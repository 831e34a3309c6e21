"""The autotuner's search and the build's use of its tuning file (CPU only)."""
import json
import os
import re

import pytest

from cumetis_gb300 import autotune as A
from cumetis_gb300 import build as B


def test_every_parameter_is_a_macro_of_its_source_with_that_default():
    for name, default, cands, src in A.PARAMS:
        text = open(os.path.join(B.CSRC, src)).read()
        m = re.search(r"#ifndef %s\s+#define %s (\d+)" % (name, name), text)
        assert m, (name, src)
        assert int(m.group(1)) == default, name
        assert default in cands, name


def test_search_reaches_the_best_valid_point_of_a_separable_cost():
    # cost: each parameter prefers one candidate; the combination TINY_MAX=16
    # with CHUNK=8192 (nine size classes) is invalid and must never be measured.
    want = {name: cands[-1] for name, _, cands, _ in A.PARAMS}
    seen = []

    def measure(cfg):
        assert A.valid(cfg)
        seen.append(dict(cfg))
        return 100.0 + sum(0.0 if cfg[n] == want[n] else 5.0 for n in cfg)

    cfg, best, trials = A.search(dict(A.DEFAULTS), measure, min_gain=0.0, log=lambda *_: None)
    assert cfg == want and best == 100.0
    assert len(trials) == len(seen)


def test_search_keeps_the_incumbent_below_the_minimum_gain():
    def measure(cfg):  # every change 0.5% faster: below a 1% threshold
        return 100.0 * (0.995 ** sum(cfg[n] != A.DEFAULTS[n] for n in cfg))

    cfg, best, _ = A.search(dict(A.DEFAULTS), measure, min_gain=0.01, log=lambda *_: None)
    assert cfg == A.DEFAULTS and best == 100.0


def test_failing_variant_is_skipped():
    def measure(cfg):
        if cfg["CM_MATCH_CHUNK"] == 512:
            raise RuntimeError("bench failed")
        return 50.0 if cfg["CM_MATCH_CHUNK"] == 128 else 60.0

    cfg, best, trials = A.search(dict(A.DEFAULTS), measure, min_gain=0.01, log=lambda *_: None)
    assert cfg["CM_MATCH_CHUNK"] == 128 and best == 50.0
    assert any(t is None for _, t in trials)


def test_defines_by_source_only_lists_changes():
    cfg = dict(A.DEFAULTS, CM_TINY_MAX=32, CM_SERIAL_DEG=8)
    assert A.defines_by_source(cfg) == {"cm_contract.cu": ["-DCM_TINY_MAX=32"],
                                        "cm_match.cu": ["-DCM_SERIAL_DEG=8"]}
    assert A.defines_by_source(dict(A.DEFAULTS)) == {}


def test_tuned_defines_from_a_tuning_file(tmp_path):
    p = tmp_path / "tuned.json"
    assert B.tuned_defines(str(p)) == []
    p.write_text(json.dumps({"defines": {"CM_TINY_MAX": 64, "CM_CHUNK": 8192}, "ms_per_step": 1.0}))
    assert B.tuned_defines(str(p)) == ["-DCM_CHUNK=8192", "-DCM_TINY_MAX=64"]
    p.write_text(json.dumps({"defines": {"CM_X; rm": 1}}))
    with pytest.raises(ValueError):
        B.tuned_defines(str(p))
