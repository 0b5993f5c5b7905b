"""Train the learned variant selector on instances the method itself labels.

Each training instance is drawn like the selector's workload (m ~ U{64..4096},
n ~ U{8..128} with m >= 2n -- the instances eligible for the mixed variants,
n <= 128 --, log10 kappa ~ U[1, 15], 5 % exactly rank deficient, 4
right-hand sides), solved on the GPU by variant 0 (Cholesky QR 2, without
its trial factor) and by variant 1 (shifted Cholesky QR 3) without fallback,
and labelled with the cheapest variant whose on-device check passed (0, else
1, else 2 = FP64 Householder).  Its features come from lila_gels_mixed_features.  The network
is trained by lila_sel_train (the library's own gradient and Adam kernels).

  python -m lila_gb300.selector_train [--instances N] [--out PATH]

writes the parameters (LILA_SEL_PARAMS float32, little endian) and a JSON
report beside them.
"""
import argparse
import ctypes
import json
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_PARAMS = os.path.join(HERE, "data", "selector_params.f32")


def label_batch(L, batch):
    """Features (count x 5 float32, device) and labels (host int32)."""
    import torch

    h = L.GelsMixed(batch.m, batch.n, batch.nrhs, batch.A_ptr, batch.lda, batch.B_ptr, batch.lda)
    F = torch.zeros((batch.count, 5), dtype=torch.float32, device="cuda")
    assert h.features(F) == 0
    _, info0, _ = h.run([0] * batch.count, flags=L.GELS_NO_FALLBACK | L.GELS_NO_TRIAL)
    batch.restore()
    _, info1, _ = h.run([1] * batch.count, flags=L.GELS_NO_FALLBACK)
    batch.restore()
    h.close()
    info0, info1 = np.asarray(info0), np.asarray(info1)
    y = np.where(info0 == 0, 0, np.where(info1 == 0, 1, 2)).astype(np.int32)
    return F, y


def load_params(path=DEFAULT_PARAMS):
    """The trained parameters as a float32 CUDA tensor (raises if absent)."""
    import torch

    p = np.fromfile(path, dtype="<f4")
    from . import lib

    if p.size != lib().lila_sel_params():
        raise RuntimeError("%s holds %d floats, expected %d" % (path, p.size, lib().lila_sel_params()))
    return torch.as_tensor(p, device="cuda")


def train(instances=1000000, batch_instances=10000, epochs=12, mb=1024, lr=2e-3, seed=5000000, log=print):
    import torch

    from . import lib
    from . import workload as W
    import lila_gb300 as L

    lib()
    feats, labels = [], []
    t0 = time.time()
    nb = (instances + batch_instances - 1) // batch_instances
    for b in range(nb):
        cnt = min(batch_instances, instances - b * batch_instances)
        batch = W.make_ls_batch(cnt, seed + b, nhi=128, klo=1.0, khi=15.0, p_rankdef=0.05)
        F, y = label_batch(L, batch)
        feats.append(F)
        labels.append(torch.as_tensor(y, device="cuda"))
        del batch
        if b % 10 == 0:
            log("batch %d/%d labelled (%.0f s)" % (b + 1, nb, time.time() - t0))
    F = torch.cat(feats)
    y = torch.cat(labels)
    n = F.shape[0]
    counts = np.bincount(y.cpu().numpy(), minlength=3)
    # hold out 5 % for the report
    perm = torch.randperm(n, generator=torch.Generator().manual_seed(1), device="cpu").to("cuda")
    nte = n // 20
    te, tr = perm[:nte], perm[nte:]
    Ftr, ytr = F[tr].contiguous(), y[tr].contiguous().to(torch.int32)
    Fte, yte = F[te].contiguous(), y[te].contiguous().to(torch.int32)
    params = torch.empty(L.lib().lila_sel_params(), dtype=torch.float32, device="cuda")
    L.sel_init(params, 7)
    cw = torch.ones(3, dtype=torch.float32, device="cuda")
    lw = L.sel_train_work(Ftr.shape[0], mb)
    work = torch.empty(lw, dtype=torch.float32, device="cuda")
    losses = (ctypes.c_float * epochs)()
    t1 = time.time()
    rc = L.sel_train(Ftr.shape[0], Ftr, ytr, cw, params, epochs, mb, lr, 11, work, lw, ctypes.addressof(losses))
    torch.cuda.synchronize()
    t_train = time.time() - t1
    assert rc == 0, rc
    choice = torch.zeros(nte, dtype=torch.int32, device="cuda")
    L.sel_infer(nte, params, Fte, None, choice)
    torch.cuda.synchronize()
    c = choice.cpu().numpy()
    yt = yte.cpu().numpy()
    conf = np.zeros((3, 3), dtype=np.int64)
    for a, b in zip(yt, c):
        conf[a, b] += 1
    report = {
        "instances": int(n), "label_counts": counts.tolist(), "epochs": epochs, "minibatch": mb, "lr": lr,
        "loss_per_epoch": [float(v) for v in losses], "train_seconds": t_train,
        "holdout": int(nte), "holdout_accuracy": float((c == yt).mean()),
        "holdout_confusion_rows_label_cols_choice": conf.tolist(),
        "label_seconds": t1 - t0,
    }
    return params, report


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--instances", type=int, default=1000000)
    ap.add_argument("--epochs", type=int, default=12)
    ap.add_argument("--out", default=DEFAULT_PARAMS)
    args = ap.parse_args()
    params, report = train(args.instances, epochs=args.epochs)
    os.makedirs(os.path.dirname(args.out), exist_ok=True)
    params.cpu().numpy().astype("<f4").tofile(args.out)
    with open(os.path.splitext(args.out)[0] + ".json", "w") as f:
        json.dump(report, f, indent=1)
    print(json.dumps(report))


if __name__ == "__main__":
    main()
