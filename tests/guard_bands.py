"""Guard-band buffers: out-of-bounds write detection without compute-sanitizer.

A guarded tensor is a view into a larger allocation whose margins (64 KiB on
each side) hold a sentinel byte; after a kernel writes the view, ``check()``
reports whether any margin byte changed, i.e. whether the kernel wrote
outside the buffer it was given.  The margins are whole multiples of 256
bytes, so a view keeps the alignment of the allocation.  Used by the GPU
guard-band tests; the helper itself is tested on the CPU.
"""
import torch

SENTINEL = 0xAD                # bytes 0xADAD.. : a tiny negative float, unlikely as a written value
PAD_BYTES = 64 * 1024


def _bytes(t):
    """Flat uint8 view of a tensor's elements (complex through its real view)."""
    if t.is_complex():
        t = torch.view_as_real(t)
    return t.reshape(-1).view(torch.uint8)


def guarded(shape, dtype, device, zero=True):
    """(view, check): ``view`` has ``shape`` and is contiguous; ``check()`` is
    True while both margins still hold the sentinel.  ``check.base`` is the
    whole allocation and ``check.pad`` the margin length in elements."""
    n = 1
    for s in shape:
        n *= int(s)
    itemsize = torch.empty((), dtype=dtype).element_size()
    pad = PAD_BYTES // itemsize
    big = torch.empty(pad + n + pad, dtype=dtype, device=device)
    raw = _bytes(big)
    raw.fill_(SENTINEL)
    body = big[pad:pad + n]
    if zero:
        body.zero_()
    lo, hi = PAD_BYTES, (pad + n) * itemsize

    def check():
        return bool((raw[:lo] == SENTINEL).all()) and bool((raw[hi:] == SENTINEL).all())

    check.base, check.pad = big, pad
    return body.view(tuple(int(s) for s in shape)), check
