"""Compute-class plumbing and argument conversion, API-compatible with freud.util
(freud/util.py:4-168)."""

from functools import wraps

import numpy as np


class _Compute:
    """Parent of all compute classes: guards access to properties before compute()."""

    def __init__(self):
        self._called_compute = False

    def __getattribute__(self, attr):
        attribute = object.__getattribute__(self, attr)
        if attr == "compute":
            compute = attribute

            @wraps(compute)
            def compute_wrapper(*args, **kwargs):
                return_value = compute(*args, **kwargs)
                self._called_compute = True
                return return_value

            return compute_wrapper
        if attr == "plot":
            if not object.__getattribute__(self, "__dict__").get("_called_compute", False):
                raise AttributeError("The compute method must be called before calling plot.")
        return attribute

    @staticmethod
    def _computed_property(prop):
        @property
        @wraps(prop)
        def wrapper(self, *args, **kwargs):
            if not self.__dict__.get("_called_compute", False):
                raise AttributeError("Property not computed. Call compute first.")
            return prop(self, *args, **kwargs)

        return wrapper

    def __str__(self):
        return repr(self)


def _convert_array(array, shape=None, dtype=np.float32, requirements=("C",), allow_copy=True):
    """Check the shape of an array and convert it to a C-contiguous array of dtype."""
    if array is None:
        return np.empty(shape, dtype=dtype)
    array = np.asarray(array)
    return_arr = np.require(array, dtype=dtype, requirements=requirements)
    if not allow_copy and return_arr is not array:
        raise ValueError("The provided output array must have dtype {}, and have the following array flags: "
                         "{}.".format(dtype, ", ".join(requirements)))
    if shape is not None:
        if return_arr.ndim != len(shape):
            raise ValueError("array.ndim = {}; expected ndim = {}".format(return_arr.ndim, len(shape)))
        for i, s in enumerate(shape):
            if s is not None and return_arr.shape[i] != s:
                shape_str = "(" + ", ".join(str(i) if i is not None else "..." for i in shape) + ")"
                raise ValueError("array.shape= {}; expected shape = {}".format(return_arr.shape, shape_str))
    return return_arr


def _convert_box(box, dimensions=None):
    """Convert a box-like object to freud_gb300.box.Box."""
    from .box import Box

    if not isinstance(box, Box):
        box = Box.from_box(box)
    if dimensions is not None and box.dimensions != dimensions:
        raise ValueError("The box must be {}-dimensional.".format(dimensions))
    return box
