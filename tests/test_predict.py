"""Node-classification evaluation (lightne_gb300.predict, the role of
LightNE/predict.py): the ShuffleSplit indices, the one-vs-rest L2 logistic
regression optimum, top-k prediction and micro/macro F1 against
scikit-learn's liblinear run of the reference's predict_cv: live where
scikit-learn is installed, and through committed scores
(tests/golden/predict_sklearn.json) on the device."""
import numpy as np
import pytest
import torch

from lightne_gb300 import predict


def _data(seed=0, n=600, d=12, L=5):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, d)).astype(np.float32)
    Wt = rng.standard_normal((d, L))
    s = X @ Wt + 0.5 * rng.standard_normal((n, L))
    Y = s > 0.8
    Y[np.arange(n), np.argmax(s, axis=1)] = True  # every node has a label
    return X, Y


def test_shuffle_splits_match_sklearn():
    sk = pytest.importorskip("sklearn.model_selection")
    for r in (0.1, 0.3, 0.9):
        ref = list(sk.ShuffleSplit(n_splits=3, test_size=1 - r, random_state=7).split(np.zeros(101)))
        got = list(predict.shuffle_splits(101, r, 3, 7))
        for (a, b), (c, d) in zip(ref, got):
            assert np.array_equal(a, c) and np.array_equal(b, d)


def test_predict_cv_matches_sklearn_liblinear():
    lm = pytest.importorskip("sklearn.linear_model")
    from sklearn.metrics import f1_score
    from sklearn.multiclass import OneVsRestClassifier
    X, Y = _data()
    got = predict.predict_cv(X, Y, train_ratio=0.3, n_splits=3, random_state=1, C=1.0, device="cpu")
    mi, ma = [], []
    for tr, te in predict.shuffle_splits(X.shape[0], 0.3, 3, 1):
        clf = OneVsRestClassifier(lm.LogisticRegression(C=1.0, solver="liblinear", tol=1e-8))
        clf.fit(X[tr], Y[tr])
        score = clf.predict_proba(X[te])
        P = predict.top_k_indicator(torch.tensor(score), torch.tensor(Y[te])).numpy()
        mi.append(f1_score(Y[te], P, average="micro"))
        ma.append(f1_score(Y[te], P, average="macro"))
    assert abs(got[0] - 100 * np.mean(mi)) < 0.5, (got, np.mean(mi))
    assert abs(got[1] - 100 * np.mean(ma)) < 0.5, (got, np.mean(ma))


def test_logistic_optimum_is_stationary():
    X, Y = _data(seed=2)
    Xt, Yt = torch.tensor(X), torch.tensor(Y)
    W = predict.fit_ovr_logistic(Xt, Yt, C=2.0)
    Xb = torch.cat([Xt.double(), torch.ones(X.shape[0], 1, dtype=torch.float64)], 1)
    ys = Yt.double() * 2 - 1
    grad = W - 2.0 * (Xb.T @ (ys * torch.sigmoid(-ys * (Xb @ W))))
    assert grad.abs().max().item() < 1e-5


def test_f1_definitions():
    Y = torch.tensor([[1, 0, 0], [0, 1, 0], [1, 1, 0]], dtype=torch.bool)
    P = torch.tensor([[1, 0, 0], [1, 0, 0], [1, 1, 0]], dtype=torch.bool)
    mi, ma = predict.f1_micro_macro(Y, P)
    assert abs(mi - 2 * 3 / (2 * 3 + 1 + 1)) < 1e-12
    assert abs(ma - (2 * 2 / 5 + 2 / 3 + 0) / 3) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("case", range(2))
def test_predict_cv_on_device_matches_sklearn_liblinear(case):
    """The device run against scikit-learn's liblinear F1 scores on the same
    data and splits (tests/golden/predict_sklearn.json, made by
    tests/golden/make_predict_golden.py), within 0.5 F1 points as on the host."""
    import json
    import os
    ref = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "predict_sklearn.json")))[case]
    X, Y = _data(seed=ref["data_seed"])
    mi, ma = predict.predict_cv(X, Y, train_ratio=ref["train_ratio"], n_splits=ref["n_splits"],
                                random_state=ref["split_seed"], C=ref["C"], device="cuda")[:2]
    assert abs(mi - ref["micro_f1"]) < 0.5, (mi, ref["micro_f1"])
    assert abs(ma - ref["macro_f1"]) < 0.5, (ma, ref["macro_f1"])


def test_predict_cv_host_matches_sklearn_fixture():
    """The same comparison on the host (no GPU), against the committed scores."""
    import json
    import os
    for ref in json.load(open(os.path.join(os.path.dirname(__file__), "golden", "predict_sklearn.json"))):
        X, Y = _data(seed=ref["data_seed"])
        mi, ma = predict.predict_cv(X, Y, train_ratio=ref["train_ratio"], n_splits=ref["n_splits"],
                                    random_state=ref["split_seed"], C=ref["C"], device="cpu")[:2]
        assert abs(mi - ref["micro_f1"]) < 0.5 and abs(ma - ref["macro_f1"]) < 0.5, (mi, ma, ref)
