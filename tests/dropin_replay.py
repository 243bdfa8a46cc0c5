"""Replay of a recorded launch_simulation_python call (src/python_interface.c
:94-192) as grav_sim's Simulator makes it (grav_sim/simulator.py:53-101):
the same arguments, each built with the ctypes type grav_sim gave it, passed
positionally to a library whose restype is set as grav_sim's
initialize_c_lib sets it (grav_sim/utils.py:51).  The recordings come from
tests/golden/make_dropin_calls.py."""
import ctypes
import json

import numpy as np

CTYPES = {"c_double": ctypes.c_double, "c_int": ctypes.c_int32, "c_bool": ctypes.c_bool,
          "c_long": ctypes.c_int64}


def replay(lib, spec, arrays, method=None):
    """Call lib.launch_simulation_python with the recorded arguments (the
    acceleration method replaced by `method` when given); returns
    (return code, ids, x, v, m) read through the returned pointers."""
    if isinstance(spec, (bytes, np.ndarray)):
        spec = json.loads(bytes(spec).decode())
    keep, args, outs = [], [], []
    num = None
    scalar_index = 0
    for a in spec:
        kind = a["kind"]
        if kind == "byref" and num is None:
            num = CTYPES[a["type"]](a["value"])
            args.append(ctypes.byref(num))
        elif kind == "byref":
            obj = CTYPES[a["type"]](a["value"])
            keep.append(obj)
            args.append(ctypes.byref(obj))
        elif kind == "array":
            dt = np.int32 if a["type"] == "c_int" else np.float64
            arr = np.ascontiguousarray(arrays[a["name"]], dtype=dt).copy()
            keep.append(arr)
            args.append(arr.ctypes.data_as(ctypes.POINTER(CTYPES[a["type"]])))
        elif kind == "out_pointer":
            p = ctypes.POINTER(CTYPES[a["type"]])()
            outs.append(p)
            args.append(ctypes.byref(p))
        elif kind == "bytes":
            args.append(a["value"].encode())
        else:
            value = a["value"]
            # scalars in grav_sim's order: G, integrator, dt, tolerance,
            # initial_dt, remove_invalid, acceleration method, ...
            if scalar_index == 6 and method is not None:
                value = method
            args.append(CTYPES[a["type"]](value))
            scalar_index += 1
    lib.launch_simulation_python.restype = ctypes.c_int
    rc = lib.launch_simulation_python(*args)
    n = num.value
    if rc != 0:
        return rc, None, None, None, None
    ids = np.ctypeslib.as_array(outs[0], shape=(n,)).copy()
    x = np.ctypeslib.as_array(outs[1], shape=(n, 3)).copy()
    v = np.ctypeslib.as_array(outs[2], shape=(n, 3)).copy()
    m = np.ctypeslib.as_array(outs[3], shape=(n,)).copy()
    return rc, ids, x, v, m
