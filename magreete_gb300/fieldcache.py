"""Field cache: a stand-in for the ``hickle`` calls of the MAGreeTe driver.

The driver caches solved fields and results with ``hkl.dump`` / ``hkl.load``
(magreete.py:391, :412, :444, :599, :637, :689, :1103; points files at
:164, :209; utils.py:808).  The cache objects are numpy arrays or lists of
arrays, e.g. ``[Ej, [alpha, k0], points, thetas]`` for a solved field
(magreete.py:391).  hickle (HDF5) is not installed in this environment, so
this module keeps the same two calls and the same objects but stores them
as a numpy ``.npz`` archive, written under exactly the file name the
driver passes (``*.hkl``): the driver's ``os.path.isfile`` checks
(magreete.py:410, :597) keep working.

Use it in place of hickle before the driver is imported:

    import sys, magreete_gb300.fieldcache as fc
    sys.modules["hickle"] = fc

It reads the files it wrote; an HDF5 file written by the real hickle raises
``ValueError`` (reading HDF5 needs h5py).
"""
from __future__ import annotations

import numpy as np

_KIND = "__fieldcache_kind__"
_HDF5_MAGIC = b"\x89HDF\r\n\x1a\n"


def _as_array(x):
    if hasattr(x, "detach"):   # torch tensor
        x = x.detach().cpu().numpy()
    return np.asarray(x)


def dump(obj, file_obj, mode="w"):
    """Write ``obj`` (an array, or a list / tuple of arrays) to ``file_obj``
    (a path, written as given, or an open binary file)."""
    if mode not in ("w", "wb"):
        raise ValueError(f"unsupported mode {mode!r}")
    if isinstance(obj, (list, tuple)):
        arrays = {f"item{i}": _as_array(x) for i, x in enumerate(obj)}
        arrays[_KIND] = np.array("list" if isinstance(obj, list) else "tuple")
    else:
        arrays = {"array": _as_array(obj), _KIND: np.array("array")}
    for k, v in arrays.items():
        if v.dtype == object:
            raise TypeError(f"entry {k} is not a numeric or string array")
    if hasattr(file_obj, "write"):
        np.savez(file_obj, **arrays)
    else:
        with open(file_obj, "wb") as f:
            np.savez(f, **arrays)


def load(file_obj):
    """Read an object written by ``dump``: the array, or the list of arrays
    (a tuple if a tuple was written)."""
    if hasattr(file_obj, "read"):
        head = file_obj.read(8)
        file_obj.seek(-len(head), 1)
    else:
        with open(file_obj, "rb") as f:
            head = f.read(8)
    if head == _HDF5_MAGIC:
        raise ValueError("HDF5 file written by hickle: this cache reads only its own .npz files")
    with np.load(file_obj, allow_pickle=False) as z:
        kind = str(z[_KIND]) if _KIND in z.files else "array"
        if kind == "array":
            return z["array"]
        items = [z[f"item{i}"] for i in range(len(z.files) - 1)]
    return items if kind == "list" else tuple(items)
