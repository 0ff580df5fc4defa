"""Observable files of the solver (stands in for the reference's HDF5 dump,
``qmctorch/utils/hdf5_utils.py:130-483``: ``dump_to_hdf5`` / ``add_group_attr``).

h5py is installed on none of the machines this package runs on, so the
store is a numpy ``.npz`` archive with the same tree: every leaf of the
dumped object is an array under ``<root>/<child>/...``, group attributes under
``<group>/@<name>``, and a root name already in the file gets the reference's
``_<n>`` suffix (hdf5_utils.py:146-157). ``load_observables`` reads a group
back as nested namespaces.
"""
from __future__ import annotations

import os
from types import SimpleNamespace

import numpy as np
import torch


def _leaves(obj, prefix, out):
    if isinstance(obj, SimpleNamespace):
        obj = vars(obj)
    if isinstance(obj, dict):
        for k, v in obj.items():
            _leaves(v, "%s/%s" % (prefix, k), out)
        return
    if isinstance(obj, torch.Tensor):
        out[prefix] = obj.detach().cpu().numpy()
        return
    if isinstance(obj, (list, tuple)) and obj and all(
            isinstance(v, (np.ndarray, torch.Tensor, float, int, np.floating)) for v in obj):
        vals = [v.detach().cpu().numpy() if isinstance(v, torch.Tensor) else np.asarray(v)
                for v in obj]
        try:
            out[prefix] = np.stack(vals)
        except ValueError:  # ragged (e.g. local energies of batches of different sizes)
            for i, v in enumerate(vals):
                out["%s/%d" % (prefix, i)] = v
        return
    if obj is None or callable(obj):
        return
    try:
        out[prefix] = np.asarray(obj)
    except Exception:
        pass


def _read(fname):
    if not os.path.exists(fname):
        return {}
    with np.load(fname, allow_pickle=False) as f:
        return {k: f[k] for k in f.files}


def _write(fname, data):
    tmp = fname + ".tmp.npz"
    np.savez(tmp, **data)
    os.replace(tmp, fname)


def dump_observables(obj, fname, root_name=None):
    """Write the leaves of ``obj`` (namespace, dict, tensors, arrays, lists)
    under ``root_name`` in the archive ``fname``; returns the root name used."""
    data = _read(fname)
    root = root_name or obj.__class__.__name__
    roots = {k.split("/")[0] for k in data}
    if root in roots:
        root = "%s_%d" % (root, sum(1 for r in roots if r.startswith(root)) + 1)
    out = {}
    _leaves(obj, root, out)
    data.update(out)
    _write(fname, data)
    return root


def add_group_attr(fname, group, attrs):
    """Attributes of a group (hdf5_utils.py add_group_attr)."""
    data = _read(fname)
    for k, v in attrs.items():
        data["%s/@%s" % (group, k)] = np.asarray(v)
    _write(fname, data)


def load_observables(fname, group):
    """The group ``group`` of the archive as nested namespaces (attributes in
    the ``attrs`` dict of the group)."""
    data = _read(fname)
    root = SimpleNamespace(attrs={})
    pre = group + "/"
    for k, v in data.items():
        if not k.startswith(pre):
            continue
        parts = k[len(pre):].split("/")
        node = root
        for p in parts[:-1]:
            if not hasattr(node, p):
                setattr(node, p, SimpleNamespace(attrs={}))
            node = getattr(node, p)
        if parts[-1].startswith("@"):
            node.attrs[parts[-1][1:]] = v
        else:
            setattr(node, parts[-1], v)
    return root
