"""Writes tests/golden/predict_sklearn.json: micro and macro F1 of
scikit-learn's liblinear one-vs-rest logistic regression (the classifier the
reference's predict.py uses, LightNE/predict.py:87-117) on the seeded data
of tests/test_predict.py, with the splits of ShuffleSplit.  The GPU test
compares lightne_gb300.predict's device run with these numbers (scikit-learn
is not installed where the GPU tests run).

    python tests/golden/make_predict_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

CASES = [  # (data seed, train ratio, splits, split seed, C)
    (3, 0.5, 2, 4, 1.0),
    (5, 0.3, 3, 9, 0.5),
]


def sklearn_f1(X, Y, ratio, n_splits, seed, C):
    import torch
    from sklearn.linear_model import LogisticRegression
    from sklearn.metrics import f1_score
    from sklearn.model_selection import ShuffleSplit
    from sklearn.multiclass import OneVsRestClassifier

    from lightne_gb300 import predict
    mi, ma = [], []
    for tr, te in ShuffleSplit(n_splits=n_splits, test_size=1 - ratio, random_state=seed).split(X):
        clf = OneVsRestClassifier(LogisticRegression(C=C, solver="liblinear", tol=1e-8))
        clf.fit(X[tr], Y[tr])
        P = predict.top_k_indicator(torch.tensor(clf.predict_proba(X[te])), torch.tensor(Y[te])).numpy()
        mi.append(f1_score(Y[te], P, average="micro"))
        ma.append(f1_score(Y[te], P, average="macro"))
    return 100 * float(np.mean(mi)), 100 * float(np.mean(ma))


def main():
    from test_predict import _data
    out = []
    for dseed, ratio, splits, sseed, C in CASES:
        X, Y = _data(seed=dseed)
        mi, ma = sklearn_f1(X, Y, ratio, splits, sseed, C)
        out.append({"data_seed": dseed, "train_ratio": ratio, "n_splits": splits, "split_seed": sseed, "C": C,
                    "micro_f1": mi, "macro_f1": ma})
    with open(os.path.join(HERE, "predict_sklearn.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
