"""Training of the frontier-scoring MLP with the engine's own CUDA kernels.

The network (in_dim -> 128 -> 128 -> 1, ReLU, sigmoid; bf16 weights, fp32
accumulation) predicts whether a search-tree extension leads to an MFI.  It is
trained on traces that the plain miner records (``Engine.mine(...,
record_trace=True)``): one row of features per created child node, label 1
when a final MFI was emitted inside that child's subtree.

PyTorch provides device memory and the stream only; forward, backward and
the Adam update are the library's kernels (sgfim_mlp_forward,
sgfim_mlp_backward, sgfim_adam_step).
"""
from __future__ import annotations

import numpy as np

FEATURES = ("prefix_support", "item_support", "extension_support", "conditional_density", "depth",
            "min_pair_cooc", "mean_pair_cooc", "sibling_position")
IN_DIM = len(FEATURES)
HIDDEN = 128


def to_bf16_bits(a):
    """float array -> uint16 bfloat16 bit patterns (round to nearest, ties to even)."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u >> 16) & 1) + 0x7FFF
    return ((u + r) >> 16).astype(np.uint16)


def from_bf16_bits(b):
    return (np.asarray(b, np.uint16).astype(np.uint32) << 16).view(np.float32)


class Trainer:
    """Holds fp32 master weights, bf16 copies and Adam moments on the GPU."""

    PARAMS = ("W1", "b1", "W2", "b2", "w3", "b3")

    def __init__(self, engine, in_dim=IN_DIM, hidden=HIDDEN, seed=0, device=0):
        import torch
        self.torch = torch
        self.eng = engine
        self.dev = torch.device(f"cuda:{device}")
        self.in_dim, self.hidden = in_dim, hidden
        rng = np.random.default_rng(seed)
        init = {
            "W1": rng.uniform(-1, 1, (hidden, in_dim)) * np.sqrt(6.0 / in_dim) / np.sqrt(2),
            "b1": np.zeros(hidden),
            "W2": rng.uniform(-1, 1, (hidden, hidden)) * np.sqrt(6.0 / hidden) / np.sqrt(2),
            "b2": np.zeros(hidden),
            "w3": rng.uniform(-1, 1, hidden) * np.sqrt(3.0 / hidden),
            "b3": np.zeros(1),
        }
        self.p = {k: torch.tensor(v, dtype=torch.float32, device=self.dev).contiguous() for k, v in init.items()}
        self.g = {k: torch.zeros_like(v) for k, v in self.p.items()}
        self.m = {k: torch.zeros_like(v) for k, v in self.p.items()}
        self.v = {k: torch.zeros_like(v) for k, v in self.p.items()}
        self.b16 = {k: torch.zeros(v.shape, dtype=torch.int16, device=self.dev) for k, v in self.p.items()
                    if k in ("W1", "W2", "w3")}
        self._refresh_bf16()
        self.steps = 0

    def _refresh_bf16(self):
        for k, t in self.b16.items():
            t.copy_(self.torch.from_numpy(to_bf16_bits(self.p[k].cpu().numpy()).view(np.int16)).to(self.dev))

    def _stream(self):
        return self.torch.cuda.current_stream(self.dev).cuda_stream

    def forward(self, X, keep=False):
        torch = self.torch
        X = X.to(self.dev, torch.float32).contiguous()
        n = X.shape[0]
        P = torch.empty(n, dtype=torch.float32, device=self.dev)
        Z1 = torch.empty((n, self.hidden), dtype=torch.float32, device=self.dev) if keep else None
        Z2 = torch.empty((n, self.hidden), dtype=torch.float32, device=self.dev) if keep else None
        self.eng.mlp_forward(X.data_ptr(), n, self.in_dim, self.hidden, self.b16["W1"].data_ptr(),
                             self.p["b1"].data_ptr(), self.b16["W2"].data_ptr(), self.p["b2"].data_ptr(),
                             self.b16["w3"].data_ptr(), self.p["b3"].data_ptr(),
                             Z1.data_ptr() if keep else 0, Z2.data_ptr() if keep else 0, P.data_ptr(),
                             self._stream())
        return (P, Z1, Z2) if keep else P

    def gradients(self, X, Y, WT=None):
        """Loss and gradients of the weighted mean BCE (fp32, on the GPU)."""
        torch = self.torch
        X = X.to(self.dev, torch.float32).contiguous()
        Y = Y.to(self.dev, torch.float32).contiguous()
        WT = WT.to(self.dev, torch.float32).contiguous() if WT is not None else None
        n = X.shape[0]
        P, Z1, Z2 = self.forward(X, keep=True)
        for t in self.g.values():
            t.zero_()
        loss = torch.zeros(1, dtype=torch.float32, device=self.dev)
        self.eng.mlp_backward(X.data_ptr(), n, self.in_dim, self.hidden, self.b16["W2"].data_ptr(),
                              self.b16["w3"].data_ptr(), Z1.data_ptr(), Z2.data_ptr(), P.data_ptr(), Y.data_ptr(),
                              WT.data_ptr() if WT is not None else 0, 1.0 / n,
                              self.g["W1"].data_ptr(), self.g["b1"].data_ptr(), self.g["W2"].data_ptr(),
                              self.g["b2"].data_ptr(), self.g["w3"].data_ptr(), self.g["b3"].data_ptr(),
                              loss.data_ptr(), self._stream())
        return loss, self.g

    def step(self, X, Y, WT=None, lr=1e-3, weight_decay=0.0):
        loss, _ = self.gradients(X, Y, WT)
        self.steps += 1
        for k in self.PARAMS:
            b16 = self.b16.get(k)
            self.eng.adam_step(self.p[k].data_ptr(), self.g[k].data_ptr(), self.m[k].data_ptr(),
                               self.v[k].data_ptr(), b16.data_ptr() if b16 is not None else 0, self.p[k].numel(),
                               lr, 0.9, 0.999, 1e-8, self.steps, weight_decay, self._stream())
        return loss

    def weights(self):
        """fp32 master weights as numpy (for sgfim_load_scorer and the oracle)."""
        return {k: v.detach().cpu().numpy().copy() for k, v in self.p.items()}

    def weights_bf16_as_float(self):
        return {k: (from_bf16_bits(self.b16[k].cpu().numpy().view(np.uint16)).astype(np.float64)
                    if k in self.b16 else self.p[k].cpu().numpy().astype(np.float64)) for k in self.PARAMS}

    def fit(self, X, Y, epochs=5, batch=4096, lr=2e-3, seed=0, balance=True):
        torch = self.torch
        X = torch.as_tensor(X, dtype=torch.float32)
        Y = torch.as_tensor(Y, dtype=torch.float32)
        n = len(X)
        WT = None
        if balance:
            pos = float(Y.sum())
            neg = n - pos
            wp = 0.5 * n / max(pos, 1.0)
            wn = 0.5 * n / max(neg, 1.0)
            WT = torch.where(Y > 0.5, torch.tensor(wp), torch.tensor(wn))
        Xd, Yd = X.to(self.dev), Y.to(self.dev)
        Wd = WT.to(self.dev) if WT is not None else None
        g = torch.Generator().manual_seed(seed)
        hist = []
        for _ in range(epochs):
            perm = torch.randperm(n, generator=g).to(self.dev)
            # the epoch's loss stays on the device: no host synchronisation per step
            tot = torch.zeros(1, dtype=torch.float32, device=self.dev)
            for a in range(0, n, batch):
                idx = perm[a:a + batch]
                loss = self.step(Xd[idx], Yd[idx], Wd[idx] if Wd is not None else None, lr=lr)
                tot += loss * len(idx)
            hist.append(float(tot.item()) / n)
        return hist
