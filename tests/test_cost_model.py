"""The cost model's CPU restatement (oracle/cost_model.py): layout and a
finite-difference check of its gradient (no GPU)."""
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def test_parameter_count_matches_header():
    from oracle import cost_model as cm
    import newman_gb300 as nm
    h = open(os.path.join(HERE, "..", "include", "newman_gb300.h")).read()
    assert int(re.search(r"#define NM_COST_PARAMS (\d+)", h).group(1)) == cm.N_PARAMS
    assert int(re.search(r"#define NM_COST_FEATURES (\d+)", h).group(1)) == cm.N_IN
    assert nm.COST_PARAMS == cm.N_PARAMS and nm.COST_FEATURES == cm.N_IN


def test_oracle_gradient_against_finite_differences():
    from oracle import cost_model as cm
    rng = np.random.default_rng(5)
    p = rng.normal(0, 0.3, cm.N_PARAMS)
    X = rng.random((40, cm.N_IN))
    T = rng.normal(0, 1, 40)
    P = cm.unpack(p, fp16=False)
    loss, g = cm.loss_and_grad(P, X, T)
    gv = cm.pack(g)
    idx = rng.choice(cm.N_PARAMS, 60, replace=False)
    h = 1e-6
    for k in idx:
        q = p.copy()
        q[k] += h
        lp, _ = cm.loss_and_grad(cm.unpack(q, fp16=False), X, T)
        q[k] -= 2 * h
        lm, _ = cm.loss_and_grad(cm.unpack(q, fp16=False), X, T)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - gv[k]) <= 1e-5 * max(1.0, abs(fd)), (k, fd, gv[k])
