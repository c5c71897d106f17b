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


MONTE_MC_STALE_SIN_PHI = 0x1
MONTE_MC_FIRST_COMPTON_Z = 0x2
MONTE_MC_NO_RAYLEIGH_TALLY = 0x4
MONTE_MC_LOCAL_MAJORANT = 0x8
class Fbp2Geom(C.Structure):
    """monte_fbp2_geom."""

    _fields_ = [
        ("n_views", C.c_int32), ("n_det", C.c_int32),
        ("view_begin", C.c_int32), ("view_end", C.c_int32),
        ("nx", C.c_int32), ("ny", C.c_int32),
        ("flags", C.c_int32), ("reserved0", C.c_int32),
        ("pitch", C.c_double), ("half", C.c_double),
        ("sod", C.c_double), ("sdd", C.c_double), ("wdist", C.c_double),
        ("pix", C.c_double), ("x0", C.c_double), ("y0", C.c_double),
        ("scale", C.c_double),
    ]


def fbp2_geom_reference():
    """recon/fbp2.cpp: 65 elements of 0.5 cm (half 16.25), 360 views of which
    1..359 are backprojected, SOD 160, SDD 220, D 60, 256^2 image at 0.1 cm
    from (-12.8, 12.8), scale 1.7, tan of degrees."""
    g = Fbp2Geom()
    g.n_views, g.n_det = 360, 65
    g.view_begin, g.view_end = 1, 360
    g.nx = g.ny = 256
    g.flags = MONTE_FDK_TAN_DEGREES
    g.pitch, g.half = 0.5, 16.25
    g.sod, g.sdd, g.wdist = 160.0, 220.0, 60.0
    g.pix, g.x0, g.y0 = 0.1, -12.8, 12.8
    g.scale = 1.7
    return g


MONTE_MC_PLAIN = 0
MONTE_MC_PERSISTENT = 1


class McGeom(C.Structure):
    """monte_mc_geom."""

    _fields_ = [
        ("n_views", C.c_int32),
        ("nu", C.c_int32),
        ("nv", C.c_int32),
        ("max_interactions", C.c_int32),
        ("flags", C.c_uint32),
        ("reserved0", C.c_int32),
        ("du", C.c_double),
        ("dv", C.c_double),
        ("half_u", C.c_double),
        ("half_v", C.c_double),
        ("sod", C.c_double),
        ("sdd", C.c_double),
        ("start_plane", C.c_double),
    ]


class McPhantom(C.Structure):
    """monte_mc_phantom (keeps references to the arrays it points at)."""

    _fields_ = [
        ("labels", C.c_void_p),
        ("nx", C.c_int32),
        ("ny", C.c_int32),
        ("nz", C.c_int32),
        ("n_labels", C.c_int32),
        ("dx", C.c_double),
        ("dy", C.c_double),
        ("dz", C.c_double),
        ("x0", C.c_double),
        ("y0", C.c_double),
        ("z0", C.c_double),
        ("clip_radius", C.c_double),
        ("clip_half_z", C.c_double),
        ("label_material", C.POINTER(C.c_int32)),
        ("label_density", C.POINTER(C.c_double)),
    ]


class McXcom(C.Structure):
    """monte_xcom."""

    _fields_ = [
        ("n_materials", C.c_int32),
        ("reserved0", C.c_int32),
        ("coherent", C.POINTER(C.c_float)),
        ("incoherent", C.POINTER(C.c_float)),
        ("photoelectric", C.POINTER(C.c_float)),
        ("total", C.POINTER(C.c_float)),
    ]


class McSpectrum(C.Structure):
    """monte_spectrum."""

    _fields_ = [
        ("n_lines", C.c_int32),
        ("reserved0", C.c_int32),
        ("energy_kev", C.POINTER(C.c_double)),
        ("weight", C.POINTER(C.c_double)),
    ]


class McRequest(C.Structure):
    """monte_mc_request."""

    _fields_ = [
        ("seed", C.c_uint64),
        ("histories_per_pixel", C.c_uint64),
        ("view_begin", C.c_int32),
        ("view_end", C.c_int32),
        ("u_begin", C.c_int32),
        ("u_end", C.c_int32),
        ("v_begin", C.c_int32),
        ("v_end", C.c_int32),
        ("kernel", C.c_int32),
        ("job", C.c_uint32),
    ]


class McStats(C.Structure):
    """monte_mc_stats."""

    _fields_ = [(n, C.c_uint64) for n in ("histories", "woodcock_steps", "interactions",
                                          "primary_counts", "scatter_counts", "dropped",
                                          "rayleigh", "compton", "photoelectric",
                                          "majorant_legs")]

    def as_dict(self):
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


def mc_geom_reference325():
    """monte_cu/CBCT_real325im.cu: 360 views, 325x325 pixels of 0.1 cm, SOD 160,
    SDD 220, start plane 10.1, 5 interactions, the stale sin_phi_a quirk."""
    g = McGeom()
    g.n_views, g.nu, g.nv = 360, 325, 325
    g.max_interactions = 5
    g.flags = MONTE_MC_STALE_SIN_PHI
    g.du = g.dv = 0.1
    g.half_u = g.half_v = 16.25
    g.sod, g.sdd, g.start_plane = 160.0, 220.0, 10.1
    return g


def mc_geom_reference_cpu():
    """monte_cpp/CBCT_real2.cpp: 65x65 pixels of 0.5 cm, start plane 6, first
    Compton about +z, no tally after Rayleigh."""
    g = McGeom()
    g.n_views, g.nu, g.nv = 360, 65, 65
    g.max_interactions = 5
    g.flags = MONTE_MC_FIRST_COMPTON_Z | MONTE_MC_NO_RAYLEIGH_TALLY
    g.du = g.dv = 0.5
    g.half_u = g.half_v = 16.25
    g.sod, g.sdd, g.start_plane = 160.0, 220.0, 6.0
    return g


def mc_geom(n_views, nu, nv, pitch_cm, sod_cm, sdd_cm, start_plane_cm, flags=0,
            max_interactions=5):
    g = McGeom()
    g.n_views, g.nu, g.nv = n_views, nu, nv
    g.max_interactions = max_interactions
    g.flags = flags
    g.du = g.dv = pitch_cm
    g.half_u = nu * pitch_cm / 2.0
    g.half_v = nv * pitch_cm / 2.0
    g.sod, g.sdd, g.start_plane = sod_cm, sdd_cm, start_plane_cm
    return g


class McInputs:
    """Host-side bundle of the phantom/XCOM/spectrum structs and the arrays
    they point at (kept alive here).  `labels` may be a numpy array (host)
    or a torch CUDA tensor (device)."""

    def __init__(self, labels, voxel_cm, origin_cm, label_material, label_density,
                 xcom_tables, energies_kev, weights=None, clip_radius=0.0, clip_half_z=0.0):
        import numpy as np
        self.labels = labels
        nz, ny, nx = labels.shape
        self.mat = np.ascontiguousarray(label_material, np.int32)
        self.rho = np.ascontiguousarray(label_density, np.float64)
        ph = McPhantom()
        ph.labels = labels.data_ptr() if hasattr(labels, "data_ptr") else labels.ctypes.data
        ph.nx, ph.ny, ph.nz = nx, ny, nz
        ph.n_labels = len(self.mat)
        ph.dx, ph.dy, ph.dz = voxel_cm if hasattr(voxel_cm, "__len__") else (voxel_cm,) * 3
        ph.x0, ph.y0, ph.z0 = origin_cm
        ph.clip_radius, ph.clip_half_z = clip_radius, clip_half_z
        ph.label_material = self.mat.ctypes.data_as(C.POINTER(C.c_int32))
        ph.label_density = self.rho.ctypes.data_as(C.POINTER(C.c_double))
        self.phantom = ph
        # xcom_tables: list of [4][201] arrays (coh, incoh, photo, total)
        tabs = np.ascontiguousarray(np.stack(xcom_tables), np.float32)  # [m][4][201]
        self.coh = np.ascontiguousarray(tabs[:, 0, :])
        self.inc = np.ascontiguousarray(tabs[:, 1, :])
        self.pho = np.ascontiguousarray(tabs[:, 2, :])
        self.tot = np.ascontiguousarray(tabs[:, 3, :])
        x = McXcom()
        x.n_materials = tabs.shape[0]
        fp = C.POINTER(C.c_float)
        x.coherent = self.coh.ctypes.data_as(fp)
        x.incoherent = self.inc.ctypes.data_as(fp)
        x.photoelectric = self.pho.ctypes.data_as(fp)
        x.total = self.tot.ctypes.data_as(fp)
        self.xcom = x
        self.E = np.ascontiguousarray(np.atleast_1d(energies_kev), np.float64)
        self.W = np.ascontiguousarray(np.ones_like(self.E) if weights is None else weights,
                                      np.float64)
        s = McSpectrum()
        s.n_lines = len(self.E)
        s.energy_kev = self.E.ctypes.data_as(C.POINTER(C.c_double))
        s.weight = self.W.ctypes.data_as(C.POINTER(C.c_double))
        self.spectrum = s


def mc_request(seed, per, views, u_range, v_range, kernel=MONTE_MC_PERSISTENT, job=0):
    r = McRequest()
    r.seed, r.histories_per_pixel = seed, per
    r.view_begin, r.view_end = views
    r.u_begin, r.u_end = u_range
    r.v_begin, r.v_end = v_range
    r.kernel, r.job = kernel, job
    return r


MONTE_BATCH_FUSED = 0
MONTE_BATCH_SEQUENTIAL = 1
MONTE_BATCH_AUTOTUNE = 0x1


class BatchJob(C.Structure):
    """monte_batch_job."""

    _fields_ = [
        ("mc", McGeom),
        ("phantom", McPhantom),
        ("spectrum", McSpectrum),
        ("seed", C.c_uint64),
        ("histories_per_pixel", C.c_uint64),
        ("fdk", FdkGeom),
        ("recon_total", C.c_int32),
        ("reserved0", C.c_int32),
        ("primary", C.c_void_p),
        ("scatter", C.c_void_p),
        ("map", C.c_void_p),
        ("vol_xy", C.c_void_p),
    ]


class SiddonGrid(C.Structure):
    """monte_siddon_grid."""

    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("reserved0", C.c_int32), ("dx", C.c_double), ("dy", C.c_double),
                ("dz", C.c_double), ("x0", C.c_double), ("y0", C.c_double),
                ("z0", C.c_double)]


def siddon_grid(shape_zyx, voxel_cm, origin_cm):
    g = SiddonGrid()
    g.nz, g.ny, g.nx = shape_zyx
    g.dx, g.dy, g.dz = voxel_cm if hasattr(voxel_cm, "__len__") else (voxel_cm,) * 3
    g.x0, g.y0, g.z0 = origin_cm
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
