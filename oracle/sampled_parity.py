"""Sampled-target parity against the CPU oracle (TEST INFRASTRUCTURE ONLY).

At the benchmark sizes (icosahedral levels 7 and 8) the oracle cannot sum every target in a
test's time, but each target of the reference's reductions is independent of the others
(src/LpmBVEKernels.hpp:163-186 BVEVertexVelocity, :285-305 BVEFaceVelocity, :140-161 and
:263-283 the stream-function functors), so a random subset of targets summed over ALL sources
checks the GPU at full size.  The subset holds vertices (distinct targets) and leaf faces
(collocated targets, the i == j pair excluded by index).

Only tests/ and bench.py's parity field use this module; it is the oracle, never the thing
measured.
"""
from __future__ import annotations

import numpy as np

from . import oracle as O


def sample_targets(nverts: int, fmask: np.ndarray, nv: int = 4096, nf: int = 4096, seed: int = 8192):
    """Sorted random vertex indices and random leaf-face indices (no masked parents)."""
    rng = np.random.default_rng(seed)
    vidx = np.sort(rng.choice(nverts, min(nv, nverts), replace=False))
    leaves = np.flatnonzero(np.asarray(fmask) == 0)
    fidx = np.sort(rng.choice(leaves, min(nf, leaves.size), replace=False))
    return vidx, fidx


def oracle_at(vx, fx, zeta, area, mask, vidx, fidx, eps=0.0):
    """Oracle velocity and stream function at the sampled vertices (distinct) and faces
    (collocated): (u_verts, psi_verts, u_faces, psi_faces)."""
    uv, pv = O.velocity_distinct(np.asarray(vx)[vidx], fx, zeta, area, mask, eps=eps, psi=True)
    uf, pf = O.velocity_faces(fidx, fx, zeta, area, mask, eps=eps, psi=True)
    return uv, pv, uf, pf


def gpu_fp64_at(ctx, P, torch, vx, fx, zeta, area, mask, vidx, fidx, eps=0.0):
    """The plain FP64 GPU path (pairFP64) at the sampled targets, through lpm_bve_velocity.

    Vertices: distinct targets over every source.  Faces: the C ABI evaluates collocated sums
    over a whole face set, so a sampled face k is summed in two calls whose source sets
    partition the unmasked faces -- (a) distinct targets x_k over every source with the sampled
    faces masked out, (b) collocated over the sampled faces alone (j != k) -- and the two FP64
    sums are added.  Device tensors in, host arrays out."""
    dev = fx.device
    vi = torch.from_numpy(np.asarray(vidx)).to(dev)
    fi = torch.from_numpy(np.asarray(fidx)).to(dev)
    f = P.FP64 | P.PSI
    uv, pv = ctx.velocity(vx[vi].contiguous(), fx, zeta, area, mask, flags=f, eps=eps)
    m2 = mask.clone()
    m2[fi] = 1
    tf = fx[fi].contiguous()
    ua, pa = ctx.velocity(tf, fx, zeta, area, m2, flags=f, eps=eps)
    ub, pb = ctx.velocity(None, tf, zeta[fi].contiguous(), area[fi].contiguous(),
                          torch.zeros(fi.numel(), dtype=torch.uint8, device=dev), flags=f | P.COLLOCATED, eps=eps)
    torch.cuda.synchronize()
    out = (uv.cpu().numpy(), pv.cpu().numpy(), (ua + ub).cpu().numpy(), (pa + pb).cpu().numpy())
    ctx.invalidate()  # these plans hold sampled copies; drop them
    return out


def _maxrel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _l2rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def compare(got, ref) -> dict:
    """max-relative (max |e| / max |ref|) and relative-L2 errors of velocity and stream
    function, vertices and faces together."""
    uv, pv, uf, pf = got
    ruv, rpv, ruf, rpf = ref
    u, ru = np.concatenate([uv, uf]), np.concatenate([ruv, ruf])
    p, rp = np.concatenate([pv, pf]), np.concatenate([rpv, rpf])
    return {"u_maxrel": _maxrel(u, ru), "u_l2": _l2rel(u, ru), "psi_maxrel": _maxrel(p, rp), "psi_l2": _l2rel(p, rp),
            "u_faces_l2": _l2rel(uf, ruf), "u_verts_l2": _l2rel(uv, ruv)}
