"""ctypes mirror of include/monte.h (structs, constants, presets).

The presets reproduce the hard-coded constants of the reference programs:
recon/bp3d20.cpp:17-19,40,85-161 and recon/bp3d20_325.cpp:17-18,43,97-171.
"""
import ctypes as C

MONTE_OK = 0
MONTE_EINVAL = -1
MONTE_ENOMEM = -2
MONTE_ECUDA = -3
MONTE_ETIMEOUT = -4
MONTE_EUNSUPPORTED = -5
MONTE_EOVERFLOW = -6

MONTE_MEM_DEVICE = 0
MONTE_MEM_HOST = 1

MONTE_FDK_TAN_DEGREES = 0x1
MONTE_FDK_FLAT_EDGE = 0x2

MONTE_FILTER_FP32 = 0
MONTE_FILTER_BF16X3 = 1
MONTE_BP_PLAIN = 0
MONTE_BP_TILED = 1


class FdkGeom(C.Structure):
    """monte_fdk_geom."""

    _fields_ = [
        ("n_views", C.c_int32),
        ("nu", C.c_int32),
        ("nv", C.c_int32),
        ("flags", C.c_int32),
        ("du", C.c_double),
        ("dv", C.c_double),
        ("half_u", C.c_double),
        ("half_v", C.c_double),
        ("sod", C.c_double),
        ("sdd", C.c_double),
        ("wdist", C.c_double),
        ("nx", C.c_int32),
        ("ny", C.c_int32),
        ("nz", C.c_int32),
        ("s_begin", C.c_int32),
        ("s_end", C.c_int32),
        ("dvox", C.c_double),
        ("x0", C.c_double),
        ("y0", C.c_double),
        ("z0", C.c_double),
        ("mask_radius", C.c_int32),
        ("reserved0", C.c_int32),
        ("scale", C.c_double),
        ("scale2", C.c_double),
    ]

    def copy(self):
        g = FdkGeom()
        C.memmove(C.byref(g), C.byref(self), C.sizeof(FdkGeom))
        return g

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


def fdk_geom_reference65():
    """recon/bp3d20.cpp: 360 views, 65x65 detector at 0.5 cm, SOD 160, SDD 220,
    weight distance 60 (:40,159), 256^3 grid at 0.1 cm, slab s in [125,130)
    (:93), sphere mask radius 118 (:145), scale 2.7 (:160)."""
    g = FdkGeom()
    g.n_views, g.nu, g.nv = 360, 65, 65
    g.flags = MONTE_FDK_TAN_DEGREES | MONTE_FDK_FLAT_EDGE
    g.du = g.dv = 0.5
    g.half_u = g.half_v = 16.25
    g.sod, g.sdd, g.wdist = 160.0, 220.0, 60.0
    g.nx = g.ny = g.nz = 256
    g.s_begin, g.s_end = 125, 130
    g.dvox = 0.1
    g.x0, g.y0, g.z0 = -12.8, 12.8, 12.8
    g.mask_radius = 118
    g.scale, g.scale2 = 2.7, 1.0
    return g


def fdk_geom_reference325():
    """recon/bp3d20_325.cpp: as bp3d20 with a 325x325 detector at 0.1 cm
    (:17,43,134-135), no sphere mask, output scaled by 2.7 then 5 (:170)."""
    g = fdk_geom_reference65()
    g.nu = g.nv = 325
    g.du = g.dv = 0.1
    g.mask_radius = 0
    g.scale, g.scale2 = 2.7, 5.0
    return g


def fdk_geom_recon325(n_views=360, nu=512, nv=384, pitch_mm=0.8, sod_mm=500.0,
                      sdd_mm=1000.0, n=325, voxel_mm=0.4):
    """FDK at the recon-325 workload: 360 views of a 512 (in-plane) x 384
    (axial) detector at 0.8 mm, SOD 500 mm, SDD 1000 mm, full 325^3 volume at
    0.4 mm (detector pitch / magnification), the reference's conventions
    otherwise (weight distance = SDD - SOD, scale 2.7, tan quirk, flat edge)."""
    g = FdkGeom()
    g.n_views, g.nu, g.nv = n_views, nu, nv
    g.flags = MONTE_FDK_TAN_DEGREES | MONTE_FDK_FLAT_EDGE
    g.du = g.dv = pitch_mm / 10.0
    g.half_u = nu * g.du / 2.0
    g.half_v = nv * g.dv / 2.0
    g.sod, g.sdd = sod_mm / 10.0, sdd_mm / 10.0
    g.wdist = g.sdd - g.sod
    g.nx = g.ny = g.nz = n
    g.s_begin, g.s_end = 0, n
    g.dvox = voxel_mm / 10.0
    c = n * g.dvox / 2.0
    g.x0, g.y0, g.z0 = -c, c, c
    g.mask_radius = 0
    g.scale, g.scale2 = 2.7, 1.0
    return g
