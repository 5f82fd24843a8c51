"""torch.autograd.Function over the C-ABI adjoint (sph_adj_*) -- used by the tests only.

``rollout(adj, x0, v0, mu, k)`` runs the adjoint's forward pass on CUDA tensors and
returns (x_T, v_T); calling .backward() on a loss of them runs sph_adj_backward and
delivers gradients to x0, v0 (float32 (n, 4) CUDA tensors) and to mu, k (float64 scalar
tensors).
"""
import torch


class SphRollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x0, v0, mu, k, adj):
        x0c = x0.detach().contiguous()
        v0c = v0.detach().contiguous()
        xT = torch.empty_like(x0c)
        vT = torch.empty_like(v0c)
        torch.cuda.synchronize()
        adj.forward(x0c.data_ptr(), v0c.data_ptr(), float(mu), float(k), out_x=xT.data_ptr(), out_v=vT.data_ptr())
        ctx.adj = adj
        ctx.scalar_like = (mu, k)
        return xT, vT

    @staticmethod
    def backward(ctx, gxT, gvT):
        gxT = gxT.contiguous()
        gvT = gvT.contiguous() if gvT is not None else None
        gx0 = torch.empty_like(gxT)
        gv0 = torch.empty_like(gxT)
        torch.cuda.synchronize()
        r = ctx.adj.backward(gxT.data_ptr(), gvT.data_ptr() if gvT is not None else None,
                             out_gx0=gx0.data_ptr(), out_gv0=gv0.data_ptr())
        mu, k = ctx.scalar_like
        g_mu = torch.tensor(r["g_mu"], dtype=mu.dtype) if torch.is_tensor(mu) else None
        g_k = torch.tensor(r["g_k"], dtype=k.dtype) if torch.is_tensor(k) else None
        return gx0, gv0, g_mu, g_k, None


def rollout(adj, x0, v0, mu, k):
    return SphRollout.apply(x0, v0, mu, k, adj)
