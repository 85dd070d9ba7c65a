"""Node-classification evaluation of an embedding on the GPU: the role of
LightNE's predict.py (LightNE/predict.py:87-117, predict_cv).

For each training ratio, the nodes are split by the same shuffles as
sklearn's ShuffleSplit(test_size = 1 - ratio, random_state = seed), a
one-vs-rest L2-regularised logistic regression is fitted per label (the
objective of liblinear's primal solver that the reference selects:
1/2 |w|^2 + C sum_i log(1 + exp(-y_i w.x_i)) with a bias feature of value 1,
regularised like the weights), every test node takes its k top-scoring
labels (k = its number of true labels, construct_indicator), and micro and
macro F1 are averaged over the splits.  The fit runs on the device as one
full-batch L-BFGS over all labels at once (the labels' problems are
independent and strictly convex, so the joint minimum is each one's).

    python -m lightne_gb300.predict --label labels.npz --embedding emb.bin --binary --dim 128 --seed 0
"""
from __future__ import annotations

import argparse
import logging
import math
import os

import numpy as np

logger = logging.getLogger(__name__)


def _torch():
    import torch
    return torch


def load_label(file: str, variable_name: str = "group"):
    """Labels as a boolean scipy CSR matrix (nodes x labels), from
    .tsv/.txt pairs, .npz, .npy or a .mat variable (predict.py:66-87)."""
    import scipy.sparse as sp
    if file.endswith(".tsv") or file.endswith(".txt"):
        data = np.loadtxt(file).astype(np.int64).reshape(-1, 2)
        return sp.csr_matrix((np.ones(data.shape[0], dtype=bool), (data[:, 0], data[:, 1])))
    if file.endswith(".npz"):
        return sp.load_npz(file).tocsr().astype(bool)
    if file.endswith(".npy"):
        return sp.csr_matrix(np.load(file)).astype(bool)
    import scipy.io
    return scipy.io.loadmat(file)[variable_name].tocsr().astype(bool)


def shuffle_splits(n: int, train_ratio: float, n_splits: int, seed: int):
    """The index splits of sklearn's ShuffleSplit(n_splits, test_size =
    1 - train_ratio, random_state = seed): one RandomState permutation per
    split, the first ceil(test_size * n) indices for testing."""
    n_test = int(math.ceil((1.0 - train_ratio) * n))
    n_train = n - n_test
    rng = np.random.RandomState(seed)
    for _ in range(n_splits):
        perm = rng.permutation(n)
        yield perm[n_test:n_test + n_train], perm[:n_test]


def fit_ovr_logistic(X, Y, C: float = 1.0, max_iter: int = 500, tol: float = 1e-7):
    """W ((d + 1) x L) minimising, for every label j,
    1/2 |w_j|^2 + C sum_i log(1 + exp(-y_ij w_j . [x_i, 1])), y in {-1, +1}.
    X, Y: device tensors (n x d float, n x L bool)."""
    torch = _torch()
    Xb = torch.cat([X, torch.ones(X.shape[0], 1, dtype=X.dtype, device=X.device)], dim=1).double()
    Ys = Y.double() * 2.0 - 1.0
    W = torch.zeros(Xb.shape[1], Y.shape[1], dtype=torch.float64, device=X.device, requires_grad=True)
    opt = torch.optim.LBFGS([W], lr=1.0, max_iter=max_iter, tolerance_grad=tol, tolerance_change=1e-14,
                            history_size=20, line_search_fn="strong_wolfe")

    def closure():
        opt.zero_grad()
        margin = Ys * (Xb @ W)
        loss = 0.5 * (W * W).sum() + C * torch.nn.functional.softplus(-margin).sum()
        loss.backward()
        return loss

    opt.step(closure)
    return W.detach()


def top_k_indicator(scores, Y):
    """Each row's k highest-scoring labels, k = its number of true labels
    (predict.py:27-42)."""
    torch = _torch()
    k = Y.sum(dim=1)
    order = torch.argsort(scores, dim=1, descending=True)
    rank = torch.empty_like(order)
    rank.scatter_(1, order, torch.arange(scores.shape[1], device=scores.device).expand_as(order))
    return rank < k[:, None]


def f1_micro_macro(Y, P):
    """Micro and macro F1 of boolean indicator matrices (labels as columns,
    as sklearn's f1_score with average='micro' / 'macro'; a label with no
    true and no predicted positives scores 0)."""
    tp = (Y & P).sum(dim=0).double()
    fp = (~Y & P).sum(dim=0).double()
    fn = (Y & ~P).sum(dim=0).double()
    micro = float(2 * tp.sum() / (2 * tp.sum() + fp.sum() + fn.sum()))
    den = 2 * tp + fp + fn
    per = torch_where(den > 0, 2 * tp / den.clamp_min(1), 0.0)
    return micro, float(per.mean())


def torch_where(cond, a, b):
    torch = _torch()
    return torch.where(cond, a, torch.as_tensor(b, dtype=a.dtype, device=a.device))


def predict_cv(X, y, train_ratio: float = 0.2, n_splits: int = 10, random_state: int = 0, C: float = 1.0,
               device: str = "cuda"):
    """Mean and std of micro / macro F1 (in %) over the splits
    (predict.py:87-117).  X: n x d array, y: n x L boolean (scipy or numpy)."""
    torch = _torch()
    Xt = torch.as_tensor(np.asarray(X, dtype=np.float32), device=device)
    Yd = y.toarray() if hasattr(y, "toarray") else np.asarray(y)
    Yt = torch.as_tensor(Yd.astype(bool), device=device)
    micro, macro = [], []
    for tr, te in shuffle_splits(Xt.shape[0], train_ratio, n_splits, random_state):
        tr_t = torch.as_tensor(tr, device=device)
        te_t = torch.as_tensor(te, device=device)
        W = fit_ovr_logistic(Xt[tr_t], Yt[tr_t], C)
        Xte = Xt[te_t].double()
        scores = torch.cat([Xte, torch.ones(Xte.shape[0], 1, dtype=Xte.dtype, device=device)], 1) @ W
        P = top_k_indicator(scores, Yt[te_t])
        mi, ma = f1_micro_macro(Yt[te_t], P)
        logger.info("micro f1 %f macro f1 %f", mi, ma)
        micro.append(mi)
        macro.append(ma)
    micro = np.array(micro) * 100
    macro = np.array(macro) * 100
    return float(np.mean(micro)), float(np.mean(macro)), float(np.std(micro)), float(np.std(macro))


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--label", required=True)
    ap.add_argument("--embedding", required=True)
    ap.add_argument("--matfile-variable-name", default="group")
    ap.add_argument("--seed", type=int, required=True)
    ap.add_argument("--start-train-ratio", type=float, default=10)
    ap.add_argument("--stop-train-ratio", type=float, default=90)
    ap.add_argument("--num-train-ratio", type=int, default=9)
    ap.add_argument("--C", type=float, default=1.0)
    ap.add_argument("--num-split", type=int, default=10)
    ap.add_argument("--dim", type=int, default=128)
    ap.add_argument("--norm", action="store_true", help="l2-normalise the embedding rows")
    ap.add_argument("--binary", action="store_true", help="raw float32 embedding (the -ne_out / -pro_out files)")
    ap.add_argument("--device", default="cuda")
    a = ap.parse_args(argv)
    logging.basicConfig(level=logging.INFO, format="%(asctime)s %(message)s")
    label = load_label(a.label, a.matfile_variable_name)
    if a.binary:
        emb = np.fromfile(a.embedding, dtype=np.float32).reshape(-1, a.dim)
    elif os.path.splitext(a.embedding)[1] == ".npy":
        emb = np.load(a.embedding)
    else:
        raise SystemExit("embedding: use --binary or a .npy file")
    keep = np.asarray(label.getnnz(axis=1) > 0).ravel()
    emb, label = emb[keep], label[keep]
    if a.norm:
        emb = emb / np.maximum(np.linalg.norm(emb, axis=1, keepdims=True), 1e-12)
    for r in np.linspace(a.start_train_ratio, a.stop_train_ratio, a.num_train_ratio):
        mi, ma, smi, sma = predict_cv(emb, label, r / 100.0, a.num_split, a.seed, a.C, a.device)
        print("train ratio %.1f%%: micro F1 %.2f (std %.2f), macro F1 %.2f (std %.2f)" % (r, mi, smi, ma, sma))


if __name__ == "__main__":
    main()
