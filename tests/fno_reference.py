"""CPU FP64 reference of the warm-start Fourier neural operator, for checking
the GPU forward and backward kernels (test infrastructure only).

Same parameter layout and the same maps as deft_gb300/csrc/fno.cu:
lift 2 -> C, L Fourier layers (truncated spectral mixing over kx, ky in
{0..m-1} U {N-m..N-1}, kz in {0..m-1}, plus a pointwise C x C map and bias,
GELU on all but the last layer), projection C -> C -> 1.  The spectral part
is written with torch.fft.rfftn / irfftn on the full grid (equal to the
truncated transforms for m < N/2), autograd gives the gradient.  Weights are
rounded to BF16 (nearest even) first, as the GPU passes use BF16 copies."""
import numpy as np
import torch


def bf16_round(x):
    a = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    a = (a + 0x7FFF + ((a >> 16) & 1)) >> 16 << 16
    return a.astype(np.uint32).view(np.float32)


def layout(C, L, m):
    Kx = Ky = 2 * m
    K = Kx * Ky * m
    off = {}
    o = 0
    off["P"] = (o, 2 * C); o += 2 * C
    off["p"] = (o, C); o += C
    for l in range(L):
        off[f"W{l}"] = (o, 2 * C * C * K); o += 2 * C * C * K
        off[f"Wp{l}"] = (o, C * C); o += C * C
        off[f"b{l}"] = (o, C); o += C
    off["Q1"] = (o, C * C); o += C * C
    off["q1"] = (o, C); o += C
    off["Q2"] = (o, C); o += C
    off["q2"] = (o, 1); o += 1
    return off, o


def loss_and_grad(params, mask, eta, target, N, C, m, L):
    """Returns (loss, y, grad) in float64 for the BF16-rounded parameters."""
    off, n = layout(C, L, m)
    assert params.size == n
    pr = torch.tensor(bf16_round(params).astype(np.float64), requires_grad=True)

    def get(name):
        o, k = off[name]
        return pr[o:o + k]

    msk = torch.tensor(np.asarray(mask, dtype=np.float64).reshape(N, N, N))
    tgt = torch.tensor(np.asarray(target, dtype=np.float64).reshape(N, N, N))
    P = get("P").view(C, 2)
    h = P[:, 0, None, None, None] * msk[None] + P[:, 1, None, None, None] * eta + \
        get("p")[:, None, None, None]
    kx = list(range(m)) + list(range(N - m, N))
    Kx = 2 * m
    for l in range(L):
        W = get(f"W{l}").view(C, C, Kx, Kx, m, 2)
        Wc = torch.complex(W[..., 0], W[..., 1])  # [i, o, kx, ky, kz]
        F = torch.fft.rfftn(h, dim=(1, 2, 3))
        V = F[:, kx][:, :, kx][:, :, :, :m]
        U = torch.einsum("ioabc,iabc->oabc", Wc, V)
        G = torch.zeros((C, N, N, N // 2 + 1), dtype=torch.complex128)
        idx = torch.tensor(kx)
        Gx = torch.zeros((C, N, Kx, m), dtype=torch.complex128).index_add(1, idx, U)
        Gxy = torch.zeros((C, N, N, m), dtype=torch.complex128).index_add(2, idx, Gx)
        G = torch.cat([Gxy, torch.zeros((C, N, N, N // 2 + 1 - m), dtype=torch.complex128)], 3)
        spec = torch.fft.irfftn(G, s=(N, N, N), dim=(1, 2, 3))
        Wp = get(f"Wp{l}").view(C, C)
        z = spec + torch.einsum("oi,ixyz->oxyz", Wp, h) + get(f"b{l}")[:, None, None, None]
        h = torch.nn.functional.gelu(z) if l < L - 1 else z
    Q1 = get("Q1").view(C, C)
    a = torch.einsum("ci,ixyz->cxyz", Q1, h) + get("q1")[:, None, None, None]
    y = torch.einsum("c,cxyz->xyz", get("Q2"), torch.nn.functional.gelu(a)) + get("q2")[0]
    loss = (msk * (y - tgt) ** 2).sum() / msk.sum()
    loss.backward()
    return float(loss.detach()), y.detach().numpy().reshape(-1), pr.grad.numpy().copy()
