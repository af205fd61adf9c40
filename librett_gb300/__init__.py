"""GB300-native tensor-transpose engine with LibreTT's plan-then-execute API.

The engine is the C++/CUDA library ``librett.so`` (include/librett.h for C++
callers, include/librett_c.h for FFI callers).  This package is a thin
Python mirror of that interface over ctypes, used by the tests and the
benchmark:

* ``librettPlan``, ``librettPlanMeasure``, ``librettExecute``,
  ``librettDestroy``, ``librettInitialize``, ``librettFinalize`` keep LibreTT's
  names, argument meaning and result codes (src/librett.h:57-121 of LibreTT);
  where C returns the handle through a pointer these return
  ``(result, handle)``.
* ``Plan`` wraps a handle and raises ``LibrettError`` on any non-success code.

Device buffers are passed as integer addresses (``tensor.data_ptr()``) and
streams as integer ``cudaStream_t`` values (``torch.cuda.Stream.cuda_stream``).
"""
from __future__ import annotations

import ctypes

from . import _lib
from ._lib import PlanInfo

LIBRETT_SUCCESS = 0
LIBRETT_INVALID_PLAN = 1
LIBRETT_INVALID_PARAMETER = 2
LIBRETT_INVALID_DEVICE = 3
LIBRETT_INTERNAL_ERROR = 4
LIBRETT_UNDEFINED_ERROR = 5

METHOD_NAMES = {0: "Unknown", 1: "Trivial", 2: "Packed", 3: "PackedSplit", 4: "Tiled",
                5: "TiledCopy"}


class LibrettError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        self.code = code
        name = _lib.load().librett_c_result_string(code).decode()
        super().__init__(f"{what}: {name}" if what else name)


def _stream(stream) -> int | None:
    if stream is None:
        return None
    if hasattr(stream, "cuda_stream"):
        return int(stream.cuda_stream)
    return int(stream)


def librettInitialize() -> None:
    _lib.load().librett_c_initialize()


def librettFinalize() -> None:
    _lib.load().librett_c_finalize()


def librettPlan(dim, permutation, sizeofType: int, stream=None) -> tuple[int, int]:
    """LibreTT librettPlan (src/librett.h:78).  Returns (result, handle)."""
    h = ctypes.c_uint(0)
    rc = _lib.load().librett_c_plan(ctypes.byref(h), len(dim), _lib.int_array(dim),
                                    _lib.int_array(permutation), sizeofType, _stream(stream))
    return rc, h.value


def librettPlanMeasure(dim, permutation, sizeofType: int, stream, idata: int,
                       odata: int) -> tuple[int, int]:
    """LibreTT librettPlanMeasure (src/librett.h:96-97).  Overwrites odata."""
    h = ctypes.c_uint(0)
    rc = _lib.load().librett_c_plan_measure(ctypes.byref(h), len(dim), _lib.int_array(dim),
                                            _lib.int_array(permutation), sizeofType,
                                            _stream(stream), idata, odata)
    return rc, h.value


def librettPlanCandidate(dim, permutation, sizeofType: int, stream,
                         candidate: int) -> tuple[int, int]:
    """Plan with one numbered candidate of the planner (no LibreTT counterpart)."""
    h = ctypes.c_uint(0)
    rc = _lib.load().librett_c_plan_candidate(ctypes.byref(h), len(dim), _lib.int_array(dim),
                                              _lib.int_array(permutation), sizeofType,
                                              _stream(stream), candidate)
    return rc, h.value


def librettExecute(handle: int, idata: int, odata: int) -> int:
    """LibreTT librettExecute (src/librett.h:121)."""
    return _lib.load().librett_c_execute(handle, idata, odata)


def librettDestroy(handle: int) -> int:
    """LibreTT librettDestroy (src/librett.h:108)."""
    return _lib.load().librett_c_destroy(handle)


def plan_info(handle: int) -> dict:
    info = PlanInfo()
    rc = _lib.load().librett_c_plan_info(handle, ctypes.byref(info))
    if rc != LIBRETT_SUCCESS:
        raise LibrettError(rc, "librett_c_plan_info")
    return info.as_dict()


def describe(dim, permutation, sizeofType: int, num_sms: int = 152,
             candidate: int = -1) -> dict:
    """Host-only planning (no device needed): what librettPlan would choose."""
    info = PlanInfo()
    rc = _lib.load().librett_c_describe(len(dim), _lib.int_array(dim),
                                        _lib.int_array(permutation), sizeofType, num_sms,
                                        candidate, ctypes.byref(info))
    if rc != LIBRETT_SUCCESS:
        raise LibrettError(rc, "librett_c_describe")
    return info.as_dict()


def transpose_noalloc(dim, permutation, sizeofType: int, stream, idata: int, odata: int) -> int:
    """One-shot transpose that allocates no device memory
    (librett_c_transpose_noalloc; no LibreTT counterpart).  Returns the
    librettResult code."""
    return _lib.load().librett_c_transpose_noalloc(len(dim), _lib.int_array(dim),
                                                   _lib.int_array(permutation), sizeofType,
                                                   _stream(stream), idata, odata)


class Group:
    """Owning wrapper of a group of plans executed as one CUDA graph
    (librett_c_group_*; no LibreTT counterpart)."""

    # policies per member size class (librett_c.h): tile + 4 * loads
    POLICY_SELECTOR, POLICY_WIDE, POLICY_WIDEST, POLICY_FILL = 0, 1, 2, 3
    LOADS_REGISTERS, LOADS_ASYNC, LOADS_PERSISTENT = 0, 4, 8

    def __init__(self, plans, idata, odata, stream=None, *, policy=None):
        n, hs, ins, outs = _handle_arrays(plans, idata, odata)
        h = ctypes.c_uint(0)
        lib = _lib.load()
        if policy is None:
            rc = lib.librett_c_group_create(ctypes.byref(h), n, hs, ins, outs, _stream(stream))
        else:
            pol = (ctypes.c_int * 12)(*expand_policy(policy))
            rc = lib.librett_c_group_create_policy(ctypes.byref(h), n, hs, ins, outs,
                                                   _stream(stream), pol)
        if rc != LIBRETT_SUCCESS:
            raise LibrettError(rc, "librett_c_group_create")
        self.handle = h.value

    def tune(self) -> None:
        """librettGroupTune: time the tile policies on this group's buffers."""
        rc = _lib.load().librett_c_group_tune(self.handle)
        if rc != LIBRETT_SUCCESS:
            raise LibrettError(rc, "librett_c_group_tune")

    def buckets(self) -> list[dict]:
        """The graph's bucket launches in launch order."""
        out = []
        lib = _lib.load()
        for b in range(self.info()["buckets"]):
            shape = (ctypes.c_int * 6)()
            m, t, by = ctypes.c_int(), ctypes.c_longlong(), ctypes.c_longlong()
            rc = lib.librett_c_group_bucket(self.handle, b, shape, ctypes.byref(m), ctypes.byref(t),
                                            ctypes.byref(by))
            if rc != LIBRETT_SUCCESS:
                raise LibrettError(rc, "librett_c_group_bucket")
            out.append({"es": shape[0], "lv": shape[1], "sv": shape[2], "nl": shape[3],
                        "smem": shape[4], "loads": shape[5], "members": m.value, "tiles": t.value,
                        "bytes": by.value})
        return out

    def policy(self) -> tuple[list[int], bool]:
        pol = (ctypes.c_int * 12)()
        tuned = ctypes.c_int(0)
        rc = _lib.load().librett_c_group_policy(self.handle, pol, ctypes.byref(tuned))
        if rc != LIBRETT_SUCCESS:
            raise LibrettError(rc, "librett_c_group_policy")
        return list(pol), bool(tuned.value)

    def execute(self) -> None:
        rc = _lib.load().librett_c_group_execute(self.handle)
        if rc != LIBRETT_SUCCESS:
            raise LibrettError(rc, "librett_c_group_execute")

    def info(self) -> dict:
        m, b, s = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        t, by = ctypes.c_longlong(), ctypes.c_longlong()
        rc = _lib.load().librett_c_group_info(self.handle, ctypes.byref(m), ctypes.byref(b),
                                              ctypes.byref(s), ctypes.byref(t), ctypes.byref(by))
        if rc != LIBRETT_SUCCESS:
            raise LibrettError(rc, "librett_c_group_info")
        return {"members": m.value, "buckets": b.value, "separate": s.value, "tiles": t.value,
                "bytes": by.value}

    def destroy(self) -> None:
        if self.handle is not None:
            _lib.load().librett_c_group_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.destroy()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def expand_policy(policy) -> list[int]:
    """A group policy per member class (12 values: size class + 4 * element-size
    index) from 1 value (all classes), 4 values (per size class, every element
    size) or 12 values."""
    p = [int(x) for x in (policy if hasattr(policy, "__len__") else [policy])]
    if len(p) == 1:
        return p * 12
    if len(p) == 4:
        return p * 3
    if len(p) == 12:
        return p
    raise ValueError("a group policy has 1, 4 or 12 values")


def _handle_arrays(plans, idata, odata):
    n = len(plans)
    if len(idata) != n or len(odata) != n:
        raise ValueError("plans, idata and odata differ in length")
    hs = (ctypes.c_uint * n)(*[p.handle if isinstance(p, Plan) else int(p) for p in plans])
    ins = (ctypes.c_void_p * n)(*[int(x) for x in idata])
    outs = (ctypes.c_void_p * n)(*[int(x) for x in odata])
    return n, hs, ins, outs


def execute_grouped(plans, idata, odata) -> None:
    """librettExecuteGrouped: one-shot grouped execution on the first plan's stream."""
    n, hs, ins, outs = _handle_arrays(plans, idata, odata)
    rc = _lib.load().librett_c_execute_grouped(n, hs, ins, outs)
    if rc != LIBRETT_SUCCESS:
        raise LibrettError(rc, "librett_c_execute_grouped")


def plan_batch(problems, stream=None, synchronize=False, timings=False):
    """librettPlan on every (dims, permutation, sizeofType) in one C call
    (librett_c_plan_batch): a list of Plan objects, with the host duration of
    each plan call in microseconds when `timings` is true."""
    n = len(problems)
    ranks = (ctypes.c_int * n)(*[len(d) for d, _, _ in problems])
    flat_d = [int(x) for d, _, _ in problems for x in d]
    flat_p = [int(x) for _, p, _ in problems for x in p]
    dims = (ctypes.c_int * max(1, len(flat_d)))(*flat_d)
    perms = (ctypes.c_int * max(1, len(flat_p)))(*flat_p)
    sizes = (ctypes.c_size_t * n)(*[int(es) for _, _, es in problems])
    hs = (ctypes.c_uint * n)()
    us = (ctypes.c_double * n)() if timings else None
    rc = _lib.load().librett_c_plan_batch(n, ranks, dims, perms, sizes, _stream(stream),
                                          1 if synchronize else 0, hs, us)
    if rc != LIBRETT_SUCCESS:
        raise LibrettError(rc, "librett_c_plan_batch")
    plans = [Plan._adopt(h, d, p, es, stream) for h, (d, p, es) in zip(hs, problems)]
    return (plans, list(us)) if timings else plans


def execute_batch(plans, idata, odata) -> None:
    """The plain per-tensor loop: librettExecute on every plan in order."""
    n, hs, ins, outs = _handle_arrays(plans, idata, odata)
    rc = _lib.load().librett_c_execute_batch(n, hs, ins, outs)
    if rc != LIBRETT_SUCCESS:
        raise LibrettError(rc, "librett_c_execute_batch")


def verify(dim, permutation, sizeofType: int, idata: int, odata: int, stream=None):
    """Device-side check of a transpose (librett_c_verify): returns (number of
    mismatching output elements, smallest mismatching output index or -1)."""
    bad, first = ctypes.c_ulonglong(0), ctypes.c_longlong(-1)
    rc = _lib.load().librett_c_verify(len(dim), _lib.int_array(dim), _lib.int_array(permutation),
                                      sizeofType, ctypes.c_void_p(idata), ctypes.c_void_p(odata),
                                      _stream(stream), ctypes.byref(bad), ctypes.byref(first))
    if rc != LIBRETT_SUCCESS:
        raise LibrettError(rc, "librett_c_verify")
    return bad.value, first.value


def launch_count() -> int:
    return int(_lib.load().librett_c_launch_count())


def table_arena_stats() -> dict:
    """Device memory the plan-table arena requested since load: slab bytes
    (cudaMalloc), table blocks handed out, bytes from its pool."""
    v = [ctypes.c_longlong(0) for _ in range(3)]
    _lib.load().librett_c_table_arena_stats(*[ctypes.byref(x) for x in v])
    return {"slab_bytes": v[0].value, "blocks": v[1].value, "pool_bytes": v[2].value}


FAULT_TABLE_ALLOC, FAULT_GROUP_ALLOC, FAULT_LAUNCH = 0, 1, 2


def inject_fault(site: int, after: int = 0) -> None:
    """Arm a host-side failure at `site` (FAULT_*): after `after` more calls
    there succeed, the next one reports a CUDA error without reaching the
    device; after < 0 disarms."""
    rc = _lib.load().librett_c_inject_fault(int(site), int(after))
    if rc != LIBRETT_SUCCESS:
        raise LibrettError(rc, "librett_c_inject_fault")


class Plan:
    """Owning wrapper of a plan handle."""

    def __init__(self, dim, permutation, sizeofType: int, stream=None, *,
                 measure: tuple[int, int] | None = None, candidate: int | None = None):
        self.dim = [int(d) for d in dim]
        self.permutation = [int(p) for p in permutation]
        self.sizeofType = int(sizeofType)
        if measure is not None:
            rc, h = librettPlanMeasure(dim, permutation, sizeofType, stream, *measure)
        elif candidate is not None:
            rc, h = librettPlanCandidate(dim, permutation, sizeofType, stream, candidate)
        else:
            rc, h = librettPlan(dim, permutation, sizeofType, stream)
        if rc != LIBRETT_SUCCESS:
            raise LibrettError(rc, "librettPlan")
        self.handle = h

    @classmethod
    def _adopt(cls, handle: int, dim, permutation, sizeofType: int, stream=None) -> "Plan":
        """A Plan owning an existing handle (from librett_c_plan_batch)."""
        self = cls.__new__(cls)
        self.dim = [int(d) for d in dim]
        self.permutation = [int(p) for p in permutation]
        self.sizeofType = int(sizeofType)
        self.handle = int(handle)
        return self

    def execute(self, idata: int, odata: int) -> None:
        rc = librettExecute(self.handle, idata, odata)
        if rc != LIBRETT_SUCCESS:
            raise LibrettError(rc, "librettExecute")

    def info(self) -> dict:
        return plan_info(self.handle)

    def status(self) -> int:
        """The plan's device status word (librett_c_plan_status): 0, or bit
        0 when a bulk-copy launch gave up waiting for its copies."""
        st = ctypes.c_uint(0)
        rc = _lib.load().librett_c_plan_status(self.handle, ctypes.byref(st))
        if rc != LIBRETT_SUCCESS:
            raise LibrettError(rc, "librett_c_plan_status")
        return st.value

    def destroy(self) -> None:
        if self.handle is not None:
            rc = librettDestroy(self.handle)
            self.handle = None
            if rc != LIBRETT_SUCCESS:
                raise LibrettError(rc, "librettDestroy")

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.destroy()

    def __del__(self):
        try:
            if getattr(self, "handle", None) is not None:
                librettDestroy(self.handle)
        except Exception:
            pass
