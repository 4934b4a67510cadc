"""Snapshot files in the reference's format (code/python/store.py:7-14 and
the trimming loop of code/python/main.py:47-52), so that runs of this
library feed the reference's plotting scripts unchanged.

`solvers.iterator` returns the reference's 100-entry list whose unset
entries are None here (empty vectors there); the reference keeps the longest
prefix whose entries all reshape to the grid, and saves it with numpy.save
as one array of shape (k, *grid, V) under
results/<problem>_<N>_<cfl>_<SPLIT>_<FLUX>_<unix time>.npy.
"""
import os
import time

import numpy as np


def snapshots(sol, shape):
    """The snapshot list of main.py:47-52: the leading set entries of the
    iterator's result, reshaped to `shape` (host numpy arrays)."""
    out = []
    for s in sol:
        if s is None:
            break
        a = s.detach().cpu().numpy() if hasattr(s, "detach") else np.asarray(s)
        if a.size != int(np.prod(shape)):
            break
        out.append(a.reshape(shape))
    return out


def result_name(T, N, cfl, SPLIT, FLUX, stamp=None):
    """<problem>_<N>_<cfl>_<SPLIT>_<FLUX>_<unix time> (store.py:12-13)."""
    name = T if isinstance(T, str) else T.__name__
    stamp = int(time.time()) if stamp is None else int(stamp)
    return "_".join(str(x) for x in [name, N, cfl, SPLIT, FLUX, stamp])


def save_results(uList, T, N, cfl, SPLIT, FLUX, directory="results", stamp=None):
    """store.py:7-14: numpy.save of the snapshot list; returns the path."""
    os.makedirs(directory, exist_ok=True)
    arrs = [u.detach().cpu().numpy() if hasattr(u, "detach") else np.asarray(u)
            for u in uList]
    path = os.path.join(directory, result_name(T, N, cfl, SPLIT, FLUX, stamp) + ".npy")
    np.save(path, np.array(arrs))
    return path
