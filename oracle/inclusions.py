"""CPU restatement of the reference's inclusion fill, for checking phono_set_inclusions.

TEST INFRASTRUCTURE ONLY (the checker of the device builder; nothing in the
product imports it).  Restates, with plain per-node loops:

  * Grid.inclusionIndices (phonomena/simulation/grid.py:158-175): for each
    target, the (y, x) nodes with sqrt((x - tx)^2 + (y - ty)^2) < r in FP64
    (float32 target fields widened), and the z selection of line 174, where
    the loop variable ``z`` is rebound to the selected index array so that
    every target after the first compares node positions, not coordinates;
  * Material.setConstants (phonomena/simulation/material.py:55-63): the
    secondary material at every selected node, in target order (later
    targets overwrite earlier ones), the primary elsewhere.

Pinned by tests/golden/materials/inclusions.npz, which holds the reference's own
result for five meshes (tests/golden/make_inclusions.py).
"""
from __future__ import annotations

import math

import numpy as np


def inclusion_ids(x, y, z, tx, ty, tz, tr, ids=None, inside=1, host=0):
    """(nx, ny, nz) uint8 material ids; ids[t] (or ``inside``) for target t."""
    x = [float(v) for v in np.asarray(x, np.float64)]
    y = [float(v) for v in np.asarray(y, np.float64)]
    zc = [float(v) for v in np.asarray(z, np.float64)]
    out = np.full((len(x), len(y), len(zc)), host, dtype=np.uint8)
    cmp = zc  # grid.py:161 binds z to the node coordinates ...
    for t in range(len(tx)):
        cx, cy, r, depth = float(np.float32(tx[t])), float(np.float32(ty[t])), float(np.float32(tr[t])), \
            float(np.float32(tz[t]))
        sel = [p for p in range(len(cmp)) if cmp[p] <= depth]
        cmp = [float(p) for p in sel]  # ... and line 174 rebinds it to the selection
        v = inside if ids is None else int(ids[t])
        for i in range(len(x)):
            for j in range(len(y)):
                dx, dy = x[i] - cx, y[j] - cy
                if math.sqrt(dx * dx + dy * dy) < r:
                    for k in sel:
                        out[i, j, k] = v
    return out
