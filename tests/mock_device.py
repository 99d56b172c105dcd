"""CPU stand-ins for the device side of the GPU package, for host-logic tests.

install(monkeypatch, pkg) routes torch's CUDA allocations to zero-filled CPU
tensors, fakes CUDA events and streams, and sends every C-ABI call through a
ctypes prototype of its declared signature (the same argument conversion as
the real call) that does nothing.  It returns the list of entry points
called.  No number computed under it means anything unless a test also
replaces the kernels it relies on.
"""
import ctypes

import torch

_REAL_DEVICE = torch.device


def _cpu(d):
    return "cpu" if d is not None and str(d).startswith("cuda") else d


class _Event:
    def __init__(self, *a, **k):
        pass

    def record(self, *a, **k):
        pass

    def elapsed_time(self, other):
        return 1.0


class _Stream:
    cuda_stream = 0


def install(monkeypatch, pkg):
    zero_for = {"empty": torch.zeros, "empty_like": torch.zeros_like}
    for name in ("zeros", "ones", "as_tensor", "tensor", "full", "arange", "zeros_like", "empty",
                 "empty_like"):
        fn = zero_for.get(name, getattr(torch, name))

        def wrapped(*a, _fn=fn, **k):
            if "device" in k:
                k["device"] = _cpu(k["device"])
            return _fn(*a, **k)
        monkeypatch.setattr(torch, name, wrapped)
    to = torch.Tensor.to

    def tensor_to(self, *a, **k):
        a = tuple(_cpu(x) if isinstance(x, (str, _REAL_DEVICE)) else x for x in a)
        if "device" in k:
            k["device"] = _cpu(k["device"])
        return to(self, *a, **k)
    monkeypatch.setattr(torch.Tensor, "to", tensor_to)
    for name, val in (("is_available", lambda: True), ("mem_get_info", lambda *a: (1 << 40, 1 << 40)),
                      ("memory_reserved", lambda *a: 0), ("memory_allocated", lambda *a: 0),
                      ("Event", _Event), ("synchronize", lambda *a: None),
                      ("current_stream", lambda *a: _Stream())):
        monkeypatch.setattr(torch.cuda, name, val)

    nat, eng = pkg._native, pkg.engine

    class TorchOnCpu:
        def __getattr__(self, n):
            return getattr(torch, n)

        def device(self, d=None, *a):
            return _REAL_DEVICE(_cpu(d) if d is not None else "cpu", *a)

    monkeypatch.setattr(eng, "_torch", lambda: TorchOnCpu())
    log = []
    protos = {}
    for name, (res, args) in nat.SIGNATURES.items():
        if res in (ctypes.c_int, ctypes.c_longlong):
            ret = (1 << 20) if res is ctypes.c_longlong else 0
            protos[name] = ctypes.CFUNCTYPE(res, *args)(lambda *a, _r=ret: _r)

    class Lib:
        def __getattr__(self, name):
            fn = protos[name]

            def g(*a):
                log.append(name)
                return fn(*a)
            return g

    def call(name, *args):
        res, argt = nat.SIGNATURES[name]
        assert len(args) == len(argt), (name, len(args), len(argt))
        log.append(name)
        return protos[name](*args)

    monkeypatch.setattr(nat, "load", lambda *a, **k: Lib())
    monkeypatch.setattr(nat, "call", call)
    return log
