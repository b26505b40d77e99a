"""ORACLE (test infrastructure only): CPU restatement of the learned smoother's per-element inputs.

Checker for the features the fused tensor-core sweep builds on the GPU (k_ml_features and
element_features_f32 in the CUDA sources). Only tests use it. The learned smoother has no
counterpart in the reference; its inputs are the ones the hot-path scope fixes for it: the 30-dof
local residual, the 10 nodal log-viscosities and 12 curved-geometry factors, per element of the two
finest multigrid levels:

* residual part: the Jacobi-scaled residual z = (r - K d) / diag(K) at the element's 10 nodes,
  divided by its Euclidean norm s (returned separately; the network's correction is scaled back by s);
* viscosity part: (log eta(node) - mu) / sigma with mu, sigma the mean and standard deviation
  (+1e-3) of log eta over all nodes of the finest level;
* geometry part: the three edge vectors from vertex 4 to vertices 1-3 divided by h = |det|^(1/3)
  (9 values), log h minus the log of the mean element size of the level (the cube root of six times
  the shell volume over the element count), the centroid radius scaled to [0, 1] across the shell,
  and the level index.
"""
from __future__ import annotations

import numpy as np


def features(levels, j, visc0, z, r_min, r_max):
    """(X [nel][52] float32, s [nel] float32) of level j in its element order."""
    f = levels[j]
    EL = np.asarray(f['EL2NOD'])
    nel = len(EL)
    X0 = levels[0]['GCOORD']                       # coarse nodes are the leading nodes of the finest level
    lv0 = np.log(np.asarray(visc0, dtype=np.float64))
    mu = lv0.mean()
    sig = np.sqrt(max((lv0 * lv0).mean() - mu * mu, 1e-12)) + 1e-3
    out = np.zeros((nel, 52), np.float32)
    zz = np.asarray(z, dtype=np.float32)[(3 * EL[:, :, None] + np.arange(3)).reshape(nel, 30)]
    s = np.sqrt(np.sum(zz.astype(np.float64) ** 2, axis=1)).astype(np.float32)
    inv = np.where(s > 0, 1.0 / np.where(s > 0, s, 1.0), 0.0).astype(np.float32)
    out[:, :30] = zz * inv[:, None]
    out[:, 30:40] = ((np.log(np.asarray(visc0, dtype=np.float64)[EL]).astype(np.float32) - np.float32(mu))
                     / np.float32(sig))
    x = X0[:, EL[:, :4]].transpose(1, 2, 0)         # (nel, 4 vertices, 3)
    ed = x[:, :3, :] - x[:, 3:4, :]
    h = np.cbrt(np.abs(np.linalg.det(ed)))
    out[:, 40:49] = (ed / h[:, None, None]).reshape(nel, 9)
    vol = 4.0 / 3.0 * np.pi * (r_max ** 3 - r_min ** 3)
    lh_ref = np.float32(np.log(np.cbrt(6.0 * vol / nel)))
    out[:, 49] = np.log(h).astype(np.float32) - lh_ref
    rc = np.sqrt(np.sum(x.mean(axis=1) ** 2, axis=1)).astype(np.float32)
    out[:, 50] = (rc - np.float32(r_min)) / (np.float32(r_max) - np.float32(r_min))
    out[:, 51] = np.float32(j)
    return out, s
