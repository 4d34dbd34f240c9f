"""Compute-class plumbing and argument conversion, API-compatible with freud.util
(freud/util.py:4-168)."""

import functools

import numpy as np


class _ComputedProperty(property):
    """A property that exists only once its object has run compute(): before
    that, reading it raises AttributeError("Property not computed. Call compute
    first."), the reference's message."""

    def __get__(self, obj, objtype=None):
        if obj is not None and not obj.__dict__.get("_has_computed", False):
            raise AttributeError("Property not computed. Call compute first.")
        return super().__get__(obj, objtype)


class _Compute:
    """Base of the compute classes. When a subclass is defined, its own compute()
    is wrapped once so that a finished call marks the object as computed; results
    are declared with _Compute._computed_property and raise AttributeError until
    then (plot(), where a subclass has one, likewise)."""

    _computed_property = _ComputedProperty

    def __init__(self):
        self._has_computed = False

    def __init_subclass__(cls, **kwargs):
        super().__init_subclass__(**kwargs)
        fn = cls.__dict__.get("compute")
        if fn is not None:
            @functools.wraps(fn)
            def compute(self, *args, **kw):
                result = fn(self, *args, **kw)
                self._has_computed = True
                return result

            cls.compute = compute
        plot = cls.__dict__.get("plot")
        if plot is not None:
            @functools.wraps(plot)
            def guarded_plot(self, *args, **kw):
                if not self.__dict__.get("_has_computed", False):
                    raise AttributeError("The compute method must be called before calling plot.")
                return plot(self, *args, **kw)

            cls.plot = guarded_plot

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
