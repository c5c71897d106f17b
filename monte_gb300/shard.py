"""Work partitioning for running the hot paths on several GPUs.

Monte Carlo: histories are independent and every history owns its random
stream, so ranks split the (view, pixel) space and the int64 tallies are
summed (the one exchange step, order-independent and bit-exact).

FDK: the filter is per view; the backprojection splits the output volume
into z-slabs, each rank needing every filtered view (all-gather of the
filtered projections), with no reduction of the volume.
"""


def split_range(n, parts, index):
    """[begin, end) of part `index` of `parts` near-equal parts of range(n)."""
    if parts <= 0 or not 0 <= index < parts:
        raise ValueError("bad part %d of %d" % (index, parts))
    q, r = divmod(n, parts)
    begin = index * q + min(index, r)
    return begin, begin + q + (1 if index < r else 0)


def mc_request_for_rank(request, n_views, rank, world):
    """Copy of a monte_mc_request restricted to this rank's views (ranks
    split the view range; a single view is split by detector columns)."""
    from .abi import McRequest
    import ctypes as C
    r = McRequest()
    C.memmove(C.byref(r), C.byref(request), C.sizeof(McRequest))
    nviews = request.view_end - request.view_begin
    if nviews >= world:
        b, e = split_range(nviews, world, rank)
        r.view_begin, r.view_end = request.view_begin + b, request.view_begin + e
    else:
        b, e = split_range(request.u_end - request.u_begin, world, rank)
        r.u_begin, r.u_end = request.u_begin + b, request.u_begin + e
    return r


def fdk_zslab_for_rank(nz, rank, world):
    """z-slab [begin, end) of the output volume owned by this rank."""
    return split_range(nz, world, rank)
