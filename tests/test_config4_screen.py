"""The batched workload's screen, repeated by the CPU oracle.

tests/golden/config4_screen.json lists which seeded candidates of the config-4
stream form the 4096-integral workload: those PAGANI converges (status 0)
within epsrel of the analytic value.  The screen was run by the GPU library;
here the oracle (the CPU restatement of the reference's iteration) repeats
the decision on a seeded sample of the candidates it finishes quickly --
accepted ones with the same region and evaluation counts, rejected ones
rejected again -- and the file's `oracle_check` entry, written by
`make_config4_screen.py --oracle-check` over every such candidate, must show
full agreement.
"""
import json

import numpy as np
import pytest

from tests.golden import make_config4_screen as S


@pytest.fixture(scope="module")
def screen():
    return json.load(open(S.PATH))


@pytest.fixture(scope="module")
def cand(screen):
    return S.candidates_of(screen)


def test_recorded_oracle_check_agrees_everywhere(screen):
    oc = screen["oracle_check"]
    assert oc["accepted_checked"] >= 3400 and oc["accepted_agree"] == oc["accepted_checked"]
    assert oc["rejected_checked"] >= 500 and oc["rejected_agree"] == oc["rejected_checked"]


def test_workload_is_the_first_accepted_candidates(screen):
    acc, rej = screen["accepted"], screen["rejected_before_last"]
    assert len(acc) == screen["target"] == 4096
    assert sorted(acc + rej) == list(range(acc[-1] + 1))


def test_oracle_repeats_accepted_sample(orc, screen, cand):
    rng = np.random.default_rng(41)
    light = [k for k, n in enumerate(screen["nregions"]) if n <= 20000]  # a second or two of CPU in all
    for k in rng.choice(light, 200, replace=False):
        ok, r = S.oracle_decision(orc, cand[screen["accepted"][k]])
        assert ok, k
        assert (r.nregions, r.neval) == (screen["nregions"][k], screen["neval"][k]), k


def test_oracle_repeats_rejected_sample(orc, screen, cand):
    rng = np.random.default_rng(43)
    low = [i for i in screen["rejected_before_last"] if cand[i].integrand.ndim <= 3]
    for i in rng.choice(low, 40, replace=False):
        ok, _ = S.oracle_decision(orc, cand[i])
        assert not ok, i
