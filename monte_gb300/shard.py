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


def fdk_views_for_rank(n_views, rank, world):
    """Views [begin, end) this rank filters before the all-gather of the
    filtered projections (the filter is per view)."""
    return split_range(n_views, world, rank)


def fdk_geom_views(g, begin, end):
    """Copy of monte_fdk_geom `g` for filtering views [begin, end) as a scan
    of their own (the cosine weights and the ramp filter do not depend on
    the view angle)."""
    from .abi import FdkGeom
    import ctypes as C
    if not 0 <= begin <= end <= g.n_views:
        raise ValueError("views [%d, %d) outside [0, %d)" % (begin, end, g.n_views))
    out = FdkGeom()
    C.memmove(C.byref(out), C.byref(g), C.sizeof(FdkGeom))
    out.n_views = end - begin
    return out


def fdk_geom_zslab(g, begin, end):
    """Copy of monte_fdk_geom `g` whose volume is slices [begin, end) of
    g's: nz = end - begin and the origin moved down by `begin` voxels
    (Z = z0 - dvox z).  The sphere mask is centred on the whole grid, which
    a slab cannot express, so masked geometries are refused."""
    from .abi import FdkGeom
    import ctypes as C
    if not 0 <= begin < end <= g.nz:
        raise ValueError("slab [%d, %d) outside [0, %d)" % (begin, end, g.nz))
    if g.mask_radius > 0:
        raise ValueError("a z-slab of a masked volume")
    out = FdkGeom()
    C.memmove(C.byref(out), C.byref(g), C.sizeof(FdkGeom))
    out.nz = end - begin
    out.z0 = g.z0 - g.dvox * begin
    return out
