"""Synthetic batched least-squares workloads (device resident).

Instances follow the least-squares driver of the reference
(least-squares/main_ls_qr3.c:94-119) at batch scale: m ~ U{mlo..mhi},
n ~ U{nlo..nhi} rejection-sampled until m >= 2n, A = U diag(sigma) V^T with
sigma_j = kappa^(-j/(n-1)), log10 kappa ~ U[klo, khi], a fraction of exactly
rank-deficient instances (sigma_n = 0), x* ~ N(0,1) (n x nrhs) and
b = A x* + noise N(0,1) * 1e-10.

Generation runs on the GPU.  U is the orthonormal factor of a seeded Gaussian
computed by Newton-Schulz iterations in FP32 on zero-padded batches (padding
rows and columns stay zero); A is then formed in FP64 from it.  U (and V)
orthonormal to FP32 accuracy perturb the singular values of A only by a
relative 1e-6, so the condition number is the requested one to six digits
even at kappa = 1e15.  V is the Q factor (sign-fixed) of a Gaussian n x n,
from a batched host QR.

Instances are grouped into chunks of similar (n, m); each chunk is one
column-major FP64 tensor of shape (count, nmax, mmax), instance t of the
chunk at offset t * nmax * mmax with leading dimension mmax, so the library
reads A_t and b_t in place.
"""
import numpy as np


class LSBatch:
    """A device-resident batch; pristine copies allow re-solving."""

    def __init__(self, m, n, kappa, rankdef, chunks, nrhs):
        self.m, self.n, self.kappa, self.rankdef = m, n, kappa, rankdef
        self.chunks = chunks  # list of dicts: idx, mmax, nmax, A, B, A0, B0, X
        self.nrhs = nrhs
        self.count = len(m)
        self.A_ptr = [0] * self.count
        self.B_ptr = [0] * self.count
        self.lda = [0] * self.count
        for ch in chunks:
            A, B = ch["A"], ch["B"]
            sa, sb = ch["nmax"] * ch["mmax"] * 8, ch["nrhs"] * ch["mmax"] * 8
            for k, t in enumerate(ch["idx"]):
                self.A_ptr[t] = A.data_ptr() + k * sa
                self.B_ptr[t] = B.data_ptr() + k * sb
                self.lda[t] = ch["mmax"]

    def restore(self):
        """Put back the pristine A and b (the FP64 solver overwrites A)."""
        for ch in self.chunks:
            ch["A"].copy_(ch["A0"])
            ch["B"].copy_(ch["B0"])

    def flops(self):
        """Householder least-squares flops (QR, Q^T b, triangular solve)."""
        m = np.asarray(self.m, dtype=np.float64)
        n = np.asarray(self.n, dtype=np.float64)
        k = self.nrhs
        return float(np.sum(2 * m * n * n - 2.0 / 3.0 * n ** 3 + k * (4 * m * n - 2 * n * n) + k * n * n))

    def bytes(self):
        m = np.asarray(self.m, dtype=np.float64)
        n = np.asarray(self.n, dtype=np.float64)
        k = self.nrhs
        return float(np.sum(8 * (m * n + k * m) + 8 * (m * n + k * n)))

    def errors(self):
        """Per instance ||x - x*|| / ||x*||, ||b - A x|| / ||b|| and ||b - A x||
        (FP64, on the device, against the pristine A and b)."""
        import torch

        fwd = np.zeros(self.count)
        res = np.zeros(self.count)
        rabs = np.zeros(self.count)
        for ch in self.chunks:
            X = ch["B"][:, :, : ch["nmax"]]  # (k, nrhs, nmax): x in rows 0..n-1
            Xs = ch["X"]
            mask_n = ch["mask_n"]  # (k, nmax)
            Xm = X * mask_n[:, None, :]
            d = torch.linalg.vector_norm((Xm - Xs).reshape(Xs.shape[0], -1), dim=1)
            s = torch.linalg.vector_norm(Xs.reshape(Xs.shape[0], -1), dim=1)
            # residual with the pristine A: B0 - A0 x  (A0 (k, nmax, mmax) = A^T rows)
            AX = torch.bmm(Xm, ch["A0"])  # (k, nrhs, mmax)
            r = torch.linalg.vector_norm((ch["B0"] - AX).reshape(Xs.shape[0], -1), dim=1)
            b = torch.linalg.vector_norm(ch["B0"].reshape(Xs.shape[0], -1), dim=1)
            idx = ch["idx"]
            fwd[idx] = (d / s).cpu().numpy()
            res[idx] = (r / b).cpu().numpy()
            rabs[idx] = r.cpu().numpy()
        return fwd, res, rabs


def _newton_schulz_rows(Y, iters=14):
    """Orthonormalise the rows of each Y[k] (n x m, zero padded) in FP32."""
    import torch

    for _ in range(iters):
        G = torch.bmm(Y, Y.transpose(1, 2))
        Y = 1.5 * Y - 0.5 * torch.bmm(G, Y)
    return Y


def make_ls_batch(count, seed, mlo=64, mhi=4096, nlo=8, nhi=128, klo=1.0, khi=12.0, p_rankdef=0.0, nrhs=4,
                  chunk=128, device="cuda"):
    import torch

    prev_tf32 = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        rng = np.random.default_rng(seed)
        m = np.zeros(count, dtype=np.int64)
        n = np.zeros(count, dtype=np.int64)
        for t in range(count):
            while True:
                mm = int(rng.integers(mlo, mhi + 1))
                nn = int(rng.integers(nlo, nhi + 1))
                if mm >= 2 * nn:
                    break
            m[t], n[t] = mm, nn
        kappa = 10.0 ** rng.uniform(klo, khi, size=count)
        rankdef = rng.random(count) < p_rankdef
        # chunks of similar n (bands of 16) and m
        order = np.lexsort((m, n // 16))
        gen = torch.Generator(device=device)
        gen.manual_seed(int(seed))
        chunks = []
        for c0 in range(0, count, chunk):
            idx = order[c0:c0 + chunk]
            k = len(idx)
            mmax = int(m[idx].max())
            mmax = (mmax + 7) // 8 * 8
            nmax = int(n[idx].max())
            mt = torch.as_tensor(m[idx], device=device)
            nt = torch.as_tensor(n[idx], device=device)
            rows = torch.arange(mmax, device=device)
            cols = torch.arange(nmax, device=device)
            mask_m = (rows[None, :] < mt[:, None]).to(torch.float32)  # (k, mmax)
            mask_n = (cols[None, :] < nt[:, None]).to(torch.float32)  # (k, nmax)
            Y = torch.randn((k, nmax, mmax), generator=gen, device=device, dtype=torch.float32)
            Y = Y * mask_m[:, None, :] * mask_n[:, :, None]
            scale = 0.95 / (torch.sqrt(mt.to(torch.float32)) + torch.sqrt(nt.to(torch.float32)))
            Y = _newton_schulz_rows(Y * scale[:, None, None])
            Y = Y.to(torch.float64)
            # V: sign-fixed Q of an n x n Gaussian, padded with the identity
            G = rng.standard_normal((k, nmax, nmax))
            for a, t in enumerate(idx):
                nn = n[t]
                G[a, nn:, :] = 0.0
                G[a, :, nn:] = 0.0
                G[a, range(nn, nmax), range(nn, nmax)] = 1.0
            Vq, Vr = np.linalg.qr(G)
            Vq = Vq * np.sign(np.diagonal(Vr, axis1=1, axis2=2))[:, None, :]
            V = torch.as_tensor(Vq, device=device, dtype=torch.float64)
            j = torch.arange(nmax, device=device, dtype=torch.float64)
            kap = torch.as_tensor(kappa[idx], device=device, dtype=torch.float64)
            nm1 = torch.clamp(nt.to(torch.float64) - 1.0, min=1.0)
            sig = torch.pow(kap[:, None], -j[None, :] / nm1[:, None]) * mask_n.to(torch.float64)
            rd = torch.as_tensor(rankdef[idx], device=device)
            last = (nt - 1).long()
            sig[rd, last[rd]] = 0.0
            # A^T = V diag(sigma) U^T  ->  column-major A with ld mmax
            A = torch.bmm(V * mask_n.to(torch.float64)[:, None, :] * mask_n.to(torch.float64)[:, :, None],
                          sig[:, :, None] * Y)
            A = A * mask_n.to(torch.float64)[:, :, None]
            Xs = torch.randn((k, nrhs, nmax), generator=gen, device=device, dtype=torch.float64)
            Xs = Xs * mask_n.to(torch.float64)[:, None, :]
            noise = torch.randn((k, nrhs, mmax), generator=gen, device=device, dtype=torch.float64)
            B = torch.bmm(Xs, A) + 1e-10 * noise * mask_m.to(torch.float64)[:, None, :]
            chunks.append({"idx": idx, "mmax": mmax, "nmax": nmax, "nrhs": nrhs, "A": A.contiguous(),
                           "B": B.contiguous(), "A0": A.clone(), "B0": B.clone(), "X": Xs,
                           "mask_n": mask_n.to(torch.float64)})
            del Y, V, G
        return LSBatch(list(map(int, m)), list(map(int, n)), kappa, rankdef, chunks, nrhs)
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev_tf32
