"""torch.autograd wrappers of the Coulomb energy and of an orbital density, for verifying the
adjoint apply and the adjoint multiply.

J(rho) = 1/2 <rho, P rho> with P the fixed-grid FP64 Poisson apply on rho's grid.  The
differentiable input is rho's vector of orthonormal coordinates on a fixed grid: the
root blocks (scaling and wavelet parts) followed by the wavelet parts of every other
node, in canonical node order.  In these coordinates the Euclidean inner product is
the L2 inner product, so the gradient is dJ/drho = 1/2 (P rho + P^T rho), computed
with mw_apply and mw_apply_adjoint.  For the symmetric kernel 1/r it equals the
potential V = P rho up to the discretisation's asymmetry.

This layer is for verification only (the gradient checks of the Coulomb energy
against V and against finite differences in the Gaussian centres); the hot path
is the C ABI.
"""
import numpy as np
import torch

import mrchem_gb300 as mw


def _cube(blocks, K):
    n = blocks.shape[0]
    b = blocks.reshape(n, 2, 2, 2, K, K, K)
    return b.transpose(0, 1, 4, 2, 5, 3, 6).reshape(n, 2 * K, 2 * K, 2 * K)


class FixedGrid:
    """A fixed grid (node keys in canonical order) with conversions tree <-> orthonormal coordinates."""

    def __init__(self, mra, keys):
        self.mra = mra
        self.K = mra.K
        self.keys = np.ascontiguousarray(keys, dtype=np.int32)
        self.root = self.keys[:, 0] == mra.root_scale
        self.index = {tuple(k): i for i, k in enumerate(self.keys)}
        self.WT = mra.basis_data()["W"].T.copy()

    @property
    def size(self):
        K3 = self.K ** 3
        return int(self.root.sum()) * 8 * K3 + int((~self.root).sum()) * 7 * K3

    def to_vec(self, tree):
        keys, coefs, _ = tree.download()
        if not np.array_equal(keys, self.keys):
            raise ValueError("tree is not on this grid")
        K3 = self.K ** 3
        return np.concatenate([coefs[self.root].ravel(), coefs[~self.root][:, K3:].ravel()])

    def to_tree(self, vec):
        """Rebuilds full blocks: scaling parts of non-root nodes by top-down reconstruction."""
        K, K3 = self.K, self.K ** 3
        n = self.keys.shape[0]
        nroot = int(self.root.sum())
        coefs = np.zeros((n, 8 * K3))
        coefs[self.root] = vec[:nroot * 8 * K3].reshape(nroot, 8 * K3)
        coefs[~self.root, K3:] = vec[nroot * 8 * K3:].reshape(n - nroot, 7 * K3)
        scales = self.keys[:, 0]
        for s in range(scales.min(), scales.max()):
            par = np.nonzero(scales == s)[0]
            par = [p for p in par if (s + 1, *(2 * self.keys[p, 1:])) in self.index]
            if not par:
                continue
            cube = _cube(coefs[par], K)
            rec = np.einsum("ai,bj,ck,nijk->nabc", self.WT, self.WT, self.WT, cube, optimize=True)
            for q, p in enumerate(par):
                for c in range(8):
                    bx, by, bz = c & 1, (c >> 1) & 1, (c >> 2) & 1
                    child = (s + 1, 2 * self.keys[p, 1] + bx, 2 * self.keys[p, 2] + by, 2 * self.keys[p, 3] + bz)
                    ci = self.index[child]
                    coefs[ci, :K3] = rec[q, bz * K:(bz + 1) * K, by * K:(by + 1) * K, bx * K:(bx + 1) * K].ravel()
        return mw.FunctionTree(self.mra).upload(self.keys, coefs)


class CoulombEnergy(torch.autograd.Function):
    """J = 1/2 <rho, P rho>; backward through the adjoint apply."""

    @staticmethod
    def forward(ctx, x, grid, oper, prec):
        rho = grid.to_tree(x.detach().cpu().numpy())
        V = mw.FunctionTree(grid.mra)
        mw.copy_grid(V, rho)
        mw.apply_fixed(prec, V, oper, rho, abs_prec=True)
        ctx.grid, ctx.oper, ctx.prec, ctx.rho, ctx.V = grid, oper, prec, rho, V
        return torch.tensor(0.5 * mw.dot(rho, V), dtype=torch.float64)

    @staticmethod
    def backward(ctx, gJ):
        grid = ctx.grid
        adj = mw.FunctionTree(grid.mra)
        mw.apply_adjoint(ctx.prec, adj, ctx.oper, ctx.rho, ctx.rho)
        g = 0.5 * (grid.to_vec(ctx.V) + grid.to_vec(adj))
        return gJ * torch.from_numpy(g), None, None, None


def coulomb_energy(x, grid, oper, prec):
    return CoulombEnergy.apply(x, grid, oper, prec)


class OrbitalDensity(torch.autograd.Function):
    """rho = occ phi^2 on a fixed grid (mw_multiply with max_iter = 0 on phi's grid); backward
    through the adjoint multiply: (d rho / d phi)^T g = 2 occ P_phi(g phi)."""

    @staticmethod
    def forward(ctx, x, grid, occ, prec):
        phi = grid.to_tree(x.detach().cpu().numpy())
        rho = mw.FunctionTree(grid.mra)
        mw.copy_grid(rho, phi)
        mw.multiply(prec, rho, occ, phi, phi, max_iter=0, abs_prec=True)
        ctx.grid, ctx.occ, ctx.prec, ctx.phi = grid, occ, prec, phi
        return torch.from_numpy(grid.to_vec(rho))

    @staticmethod
    def backward(ctx, g):
        grid = ctx.grid
        seed = grid.to_tree(g.detach().cpu().numpy())
        adj = mw.FunctionTree(grid.mra)
        mw.multiply_adjoint(ctx.prec, adj, 2.0 * ctx.occ, ctx.phi, ctx.phi, seed)
        return torch.from_numpy(grid.to_vec(adj)), None, None, None


def orbital_density(x, grid, occ, prec):
    return OrbitalDensity.apply(x, grid, occ, prec)
