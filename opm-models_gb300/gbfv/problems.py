"""Problem descriptions: grids, rock, fluids, boundaries and constraints as
plain numpy arrays, packed into the ``gbfv_problem`` C struct.

The builders restate the reference's test problems as input specifications:
  * ``lens``      -- tests/problems/lensproblem.hh:227-627 (2D 48x32 DNAPL
                     infiltration with a low-permeability lens)
  * ``blackoil``  -- tests/problems/reservoirproblem.hh:215-736 with the
                     synthetic changes of the 3-phase benchmark: lognormal
                     permeability, uniform porosity, 10-row PVT tables, Corey
                     relperms, corner wells as constraint cells
  * ``ensemble_member`` -- 3D two-phase lens-like realisations for batching

Grids are YaspGrid-like: cell index i + nx*(j + ny*k), intersections in the
order -x,+x,-y,+y,-z,+z (dirId 0..5, ecfvstencil.hh:150-165).
"""
import ctypes as C
import math

import numpy as np

from . import capi

# reservoirproblem.hh:223-279 (saturated live-oil and dry-gas tables)
REF_BO = [(101353, 1.062), (1.82504e+06, 1.15), (3.54873e+06, 1.207), (6.99611e+06, 1.295),
          (1.38909e+07, 1.435), (1.73382e+07, 1.5), (2.07856e+07, 1.565), (2.76804e+07, 1.695),
          (3.45751e+07, 1.827)]
REF_MUO = [(101353, 0.00104), (1.82504e+06, 0.000975), (3.54873e+06, 0.00091),
           (6.99611e+06, 0.00083), (1.38909e+07, 0.000695), (1.73382e+07, 0.000641),
           (2.07856e+07, 0.000594), (2.76804e+07, 0.00051), (3.45751e+07, 0.000449)]
REF_RS = [(101353, 0.178108), (1.82504e+06, 16.1187), (3.54873e+06, 32.0594),
          (6.99611e+06, 66.0779), (1.38909e+07, 113.276), (1.73382e+07, 138.033),
          (2.07856e+07, 165.64), (2.76804e+07, 226.197), (3.45751e+07, 288.178)]
REF_BG = [(101353, 0.93576), (1.82504e+06, 0.0678972), (3.54873e+06, 0.0352259),
          (6.99611e+06, 0.0179498), (1.38909e+07, 0.00906194), (1.73382e+07, 0.00726527),
          (2.07856e+07, 0.00606375), (2.76804e+07, 0.00455343), (3.45751e+07, 0.00364386),
          (6.21542e+07, 0.00216723)]
REF_MUG = [(101353, 8e-06), (1.82504e+06, 9.6e-06), (3.54873e+06, 1.12e-05), (6.99611e+06, 1.4e-05),
           (1.38909e+07, 1.89e-05), (1.73382e+07, 2.08e-05), (2.07856e+07, 2.28e-05),
           (2.76804e+07, 2.68e-05), (3.45751e+07, 3.09e-05), (6.21542e+07, 4.7e-05)]


class ProblemData:
    """Owns the numpy arrays behind one ``gbfv_problem``."""

    def __init__(self, model):
        self.model = model
        self.b = 3 if model == capi.MODEL_BLACKOIL_3P else 2
        self.gravity = (0.0, 0.0, 0.0)
        self.rho = (0.0, 0.0)
        self.mu = (0.0, 0.0)
        self.pvt_arrays = None
        self.constraint = None
        self.constraint_pv = np.zeros(0)
        self.constraint_meaning = np.zeros(0, np.int32)
        self.init_pv = None
        self.init_meaning = None
        self.temperature = 293.15
        self.info = {}
        self.flux_module = capi.FLUX_DARCY

    @property
    def num_cells(self):
        return len(self.volume)

    def struct(self):
        """Build the C struct; the returned object keeps references alive."""
        s = capi.Problem()
        s.model = self.model
        s.num_cells = self.num_cells
        s.num_conn = len(self.conn_nbr)
        s.num_bfaces = len(self.bface_area)
        D, I = C.c_double, C.c_int32
        s.center = capi.as_ptr(self.center, D)
        s.volume = capi.as_ptr(self.volume, D)
        s.porosity = capi.as_ptr(self.porosity, D)
        s.perm = capi.as_ptr(self.perm, D)
        s.material = capi.as_ptr(self.material, I)
        s.conn_ptr = capi.as_ptr(self.conn_ptr, I)
        s.conn_nbr = capi.as_ptr(self.conn_nbr, I)
        s.conn_dir = capi.as_ptr(self.conn_dir, I)
        s.conn_normal = capi.as_ptr(self.conn_normal, D)
        s.conn_center = capi.as_ptr(self.conn_center, D)
        s.conn_area = capi.as_ptr(self.conn_area, D)
        s.bface_ptr = capi.as_ptr(self.bface_ptr, I)
        s.bface_normal = capi.as_ptr(self.bface_normal, D)
        s.bface_center = capi.as_ptr(self.bface_center, D)
        s.bface_area = capi.as_ptr(self.bface_area, D)
        s.bface_type = capi.as_ptr(self.bface_type, I)
        s.bface_value = capi.as_ptr(self.bface_value, D)
        s.constraint = capi.as_ptr(self.constraint, I)
        s.num_constraints = len(self.constraint_meaning)
        s.constraint_pv = capi.as_ptr(self.constraint_pv if len(self.constraint_pv) else None, D)
        s.constraint_meaning = capi.as_ptr(
            self.constraint_meaning if len(self.constraint_meaning) else None, I)
        s.gravity = (C.c_double * 3)(*self.gravity)
        s.num_materials = len(self.material_params) // capi.MAT_STRIDE
        s.material_params = capi.as_ptr(self.material_params, D)
        s.rho = (C.c_double * 2)(*self.rho)
        s.mu = (C.c_double * 2)(*self.mu)
        s.temperature = self.temperature
        s.flux_module = self.flux_module
        ec = getattr(self, "elem_corner", None)
        if ec is not None:
            s.num_elements = len(ec) // 4
            s.elem_corner = capi.as_ptr(ec, I)
            s.bface_corner = capi.as_ptr(self.bface_corner, I)
            s.p1_gradients = self.p1_gradients
        if self.pvt_arrays is not None:
            a = self.pvt_arrays
            pv = capi.BlackOilPvt()
            pv.rho_ref_oil, pv.rho_ref_water, pv.rho_ref_gas = a["rho_ref"]
            pv.n_oil = len(a["oil_p"])
            pv.oil_p = capi.as_ptr(a["oil_p"], D)
            pv.oil_rs = capi.as_ptr(a["oil_rs"], D)
            pv.oil_bo = capi.as_ptr(a["oil_bo"], D)
            pv.oil_mu = capi.as_ptr(a["oil_mu"], D)
            pv.oil_compressibility = a["oil_comp"]
            pv.n_gas = len(a["gas_p"])
            pv.gas_p = capi.as_ptr(a["gas_p"], D)
            pv.gas_bg = capi.as_ptr(a["gas_bg"], D)
            pv.gas_mu = capi.as_ptr(a["gas_mu"], D)
            pv.water_p_ref = a["water_p_ref"]
            pv.water_bw_ref = a["water_bw_ref"]
            pv.water_compressibility = a["water_comp"]
            pv.water_mu = a["water_mu"]
            self._pvt_struct = pv
            s.pvt = C.pointer(pv)
        else:
            s.pvt = C.cast(None, C.POINTER(capi.BlackOilPvt))
        self._struct = s
        return s


def structured_grid(nx, ny, nz, lx, ly, lz, dim):
    """Cell and intersection arrays of an axis-aligned Cartesian grid."""
    if dim == 2:
        nz = 1
    hx, hy = lx / nx, ly / ny
    hz = lz / nz if dim == 3 else 1.0
    N = nx * ny * nz
    idx = np.arange(N)
    i = idx % nx
    j = (idx // nx) % ny
    k = idx // (nx * ny)
    center = np.zeros((N, 3))
    center[:, 0] = (i + 0.5) * hx
    center[:, 1] = (j + 0.5) * hy
    if dim == 3:
        center[:, 2] = (k + 0.5) * hz
    vol = hx * hy * (hz if dim == 3 else 1.0)
    volume = np.full(N, vol)
    h = [hx, hy, hz]
    area_of = [hy * (hz if dim == 3 else 1.0), hx * (hz if dim == 3 else 1.0), hx * hy]
    # intersections in order -x,+x,-y,+y,-z,+z
    coords = [i, j, k]
    ns = [nx, ny, nz]
    strides = [1, nx, nx * ny]
    ndir = 2 * dim
    has_nbr = np.zeros((N, ndir), bool)
    nbr = np.full((N, ndir), -1, np.int64)
    for d in range(dim):
        lo = coords[d] > 0
        hi = coords[d] < ns[d] - 1
        has_nbr[:, 2 * d] = lo
        has_nbr[:, 2 * d + 1] = hi
        nbr[lo, 2 * d] = idx[lo] - strides[d]
        nbr[hi, 2 * d + 1] = idx[hi] + strides[d]
    normals = np.zeros((ndir, 3))
    for d in range(dim):
        normals[2 * d, d] = -1.0
        normals[2 * d + 1, d] = 1.0
    # flatten interior connections per cell in intersection order
    cnt = has_nbr.sum(1)
    conn_ptr = np.zeros(N + 1, np.int64)
    np.cumsum(cnt, out=conn_ptr[1:])
    cells, dirs = np.nonzero(has_nbr)
    conn_nbr = nbr[cells, dirs]
    conn_normal = normals[dirs]
    conn_center = center[cells].copy()
    off = np.where(dirs % 2 == 0, -0.5, 0.5)
    for d in range(dim):
        m = dirs // 2 == d
        conn_center[m, d] += off[m] * h[d]
    conn_area = np.array([area_of[d // 2] for d in range(ndir)])[dirs]
    bcnt = (~has_nbr).sum(1)
    bface_ptr = np.zeros(N + 1, np.int64)
    np.cumsum(bcnt, out=bface_ptr[1:])
    bcells, bdirs = np.nonzero(~has_nbr)
    bface_normal = normals[bdirs]
    bface_center = center[bcells].copy()
    boff = np.where(bdirs % 2 == 0, -0.5, 0.5)
    for d in range(dim):
        m = bdirs // 2 == d
        bface_center[m, d] += boff[m] * h[d]
    bface_area = np.array([area_of[d // 2] for d in range(ndir)])[bdirs]
    return dict(nx=nx, ny=ny, nz=nz, dim=dim, N=N, center=center, volume=volume,
                conn_ptr=conn_ptr.astype(np.int32), conn_nbr=conn_nbr.astype(np.int32),
                conn_dir=dirs.astype(np.int32), conn_normal=conn_normal,
                conn_center=conn_center, conn_area=conn_area,
                bface_ptr=bface_ptr.astype(np.int32), bface_cell=bcells.astype(np.int32),
                bface_dir=bdirs.astype(np.int32), bface_normal=bface_normal,
                bface_center=bface_center, bface_area=bface_area,
                bbox_min=np.zeros(3), bbox_max=np.array([lx, ly, lz if dim == 3 else 0.0]))


def _fill_grid(p, g):
    p.grid = g
    p.center = np.ascontiguousarray(g["center"].ravel())
    p.volume = g["volume"]
    p.conn_ptr = g["conn_ptr"]
    p.conn_nbr = g["conn_nbr"]
    p.conn_dir = g["conn_dir"]
    p.conn_normal = np.ascontiguousarray(g["conn_normal"].ravel())
    p.conn_center = np.ascontiguousarray(g["conn_center"].ravel())
    p.conn_area = g["conn_area"]
    p.bface_ptr = g["bface_ptr"]
    p.bface_normal = np.ascontiguousarray(g["bface_normal"].ravel())
    p.bface_center = np.ascontiguousarray(g["bface_center"].ravel())
    p.bface_area = g["bface_area"]


def vg_params(swr, snr, alpha, n):
    return [capi.LAW_REG_VAN_GENUCHTEN, swr, snr, alpha, n, 0, 0, 0]


def bc_params(swr, snr, pe, lam):
    return [capi.LAW_REG_BROOKS_COREY, swr, snr, pe, lam, 0, 0, 0]


def lens(nx=48, ny=32, law="vg", dim=2, nz=16, flux="darcy"):
    """LensProblem (lensproblem.hh:227-627), default 2D 48x32 over 6 m x 4 m;
    flux="trans" selects the transmissibility flux module
    (lens_immiscible_ecfv_ad_trans.cc:55-58)."""
    lx, ly, lz = 6.0, 4.0, 1.0
    g = structured_grid(nx, ny, nz, lx, ly, lz, dim)
    p = ProblemData(capi.MODEL_IMMISCIBLE_2P)
    _fill_grid(p, g)
    N = g["N"]
    eps = 3e-6
    lens_ll = np.array([1.0, 2.0, 0.0])
    lens_ur = np.array([4.0, 3.0, 1.0])
    c = g["center"]
    in_lens = np.ones(N, bool)
    for d in range(dim):
        in_lens &= (c[:, d] >= lens_ll[d] - eps) & (c[:, d] <= lens_ur[d] + eps)
    p.material = np.where(in_lens, 1, 0).astype(np.int32)
    kl, ko = 9.05e-12, 4.6e-10
    p.perm = np.ascontiguousarray(np.repeat(np.where(in_lens, kl, ko)[:, None], 3, 1).ravel())
    p.porosity = np.full(N, 0.4)
    if law == "vg":
        mats = vg_params(0.05, 0.0, 0.0037, 4.7) + vg_params(0.18, 0.0, 0.00045, 7.3)
    else:
        mats = bc_params(0.05, 0.0, 500.0, 2.0) + bc_params(0.18, 0.0, 2000.0, 2.0)
    p.material_params = np.array(mats, float)
    # SimpleH2O / DNAPL liquids
    p.rho = (1000.0, 1460.0)
    p.mu = (1e-3, 5.7e-4)
    vert = 1 if dim == 2 else 2  # index of the vertical axis
    grav = [0.0, 0.0, 0.0]
    grav[vert] = -9.81
    p.gravity = tuple(grav)
    p.temperature = 273.15 + 20
    # boundary conditions (lensproblem.hh:468-537)
    ymax = ly if dim == 2 else lz
    btype, bval = _lens_boundary(g["bface_center"], lx, ymax, vert, p.rho[0], grav[vert])
    p.bface_type = btype
    p.bface_value = np.ascontiguousarray(bval.ravel())
    p.constraint = np.full(N, -1, np.int32)
    # initial condition (lensproblem.hh:549-582)
    p.init_pv = _lens_initial(c, ymax, vert, p.rho[0], grav[vert])
    p.init_meaning = np.zeros(N, np.int32)
    p.info = dict(name="lens", nx=nx, ny=ny, nz=(nz if dim == 3 else 1), dim=dim, flux=flux)
    if flux == "trans":
        p.flux_module = capi.FLUX_TRANS
    elif flux != "darcy":
        raise ValueError("flux must be 'darcy' or 'trans'")
    return p


def _lens_boundary(positions, xmax, ymax, vert, rho_w, gy, eps=3e-6):
    """LensProblem::boundary (lensproblem.hh:468-537) at each boundary
    integration point: free flow (hydrostatic p_w, S_w = 1; scaled by
    1 + 1.5/height on the left) on the left and right, the NAPL inlet on the
    top for 0.5 < lambda < 2/3, no flow elsewhere."""
    nb = len(positions)
    btype = np.zeros(nb, np.int32)
    bval = np.zeros((nb, 4))
    xmin = 0.0
    height = ymax
    for f in range(nb):
        pos = positions[f]
        on_left = pos[0] < xmin + eps
        on_right = pos[0] > xmax - eps
        on_upper = pos[vert] > ymax - eps
        width = xmax - xmin
        lam = (xmax - pos[0]) / width
        if on_left or on_right:
            depth = ymax - pos[vert]
            if on_left:
                alpha = (1 + 1.5 / height)
                pw = 1e5 - alpha * rho_w * gy * depth
            else:
                pw = 1e5 - rho_w * gy * depth
            btype[f] = capi.BC_FREEFLOW
            bval[f, 0] = pw
            bval[f, 1] = 1.0
        elif on_upper and 0.5 < lam < 2.0 / 3.0:
            btype[f] = capi.BC_MASSRATE
            bval[f, 1] = -0.04
    return btype, bval


def _lens_initial(positions, ymax, vert, rho_w, gy):
    """LensProblem::initial (lensproblem.hh:549-582): hydrostatic p_w, S_w = 1."""
    depth = ymax - positions[:, vert]
    pw = 1e5 - rho_w * gy * depth
    return np.ascontiguousarray(np.stack([pw, np.ones(len(positions))], 1).ravel())


def _quad_area(p0, p1, p2, p3):
    """Area of the quadrilateral p0 p1 p2 p3 (VcfvStencil::quadrilateralArea,
    vcfvstencil.hh:495-501)."""
    return 0.5 * abs((p3[0] - p1[0]) * (p2[1] - p0[1]) - (p3[1] - p1[1]) * (p2[0] - p0[0]))


# 2D cube reference element (dune-geometry numbering): corner c at
# ((c & 1), (c >> 1) & 1); face f: 0 x = 0, 1 x = 1, 2 y = 0, 3 y = 1, with
# corners FACE_CORNERS[f] and centre FACE_CENTER[f]
FACE_CORNERS = ((0, 2), (1, 3), (0, 1), (2, 3))
FACE_CENTER = ((0.0, 0.5), (1.0, 0.5), (0.5, 0.0), (0.5, 1.0))
FACE_NORMAL = ((-1.0, 0.0), (1.0, 0.0), (0.0, -1.0), (0.0, 1.0))


def lens_vcfv(nx=48, ny=32, law="vg", p1=True):
    """LensProblem on the vertex-centred discretization
    (lens_immiscible_vcfv_ad.cc / lens_immiscible_vcfv_fd.cc: 2D 48x32
    elements over 6 m x 4 m, P1 finite-element gradients).  The degrees of
    freedom are the (nx+1) x (ny+1) vertices, index i + (nx+1) j; element
    ex + nx ey has corners (ex, ey), (ex+1, ey), (ex, ey+1), (ex+1, ey+1).
    Material, permeability and the initial state are the problem's at each
    vertex; boundary conditions at each boundary sub-control-volume face's
    integration point (half way from the corner to the intersection's
    centre, vcfvstencil.hh:966-1010)."""
    lx, ly = 6.0, 4.0
    hx, hy = lx / nx, ly / ny
    mx, my = nx + 1, ny + 1
    N = mx * my
    vi = np.arange(N)
    pos = np.zeros((N, 3))
    pos[:, 0] = (vi % mx) * hx
    pos[:, 1] = (vi // mx) * hy
    p = ProblemData(capi.MODEL_IMMISCIBLE_2P)
    p.center = np.ascontiguousarray(pos.ravel())
    eps = 3e-6
    lens_ll, lens_ur = (1.0, 2.0), (4.0, 3.0)
    in_lens = np.ones(N, bool)
    for d in range(2):
        in_lens &= (pos[:, d] >= lens_ll[d] - eps) & (pos[:, d] <= lens_ur[d] + eps)
    p.material = np.where(in_lens, 1, 0).astype(np.int32)
    kl, ko = 9.05e-12, 4.6e-10
    p.perm = np.ascontiguousarray(np.repeat(np.where(in_lens, kl, ko)[:, None], 3, 1).ravel())
    p.porosity = np.full(N, 0.4)
    if law == "vg":
        mats = vg_params(0.05, 0.0, 0.0037, 4.7) + vg_params(0.18, 0.0, 0.00045, 7.3)
    else:
        mats = bc_params(0.05, 0.0, 500.0, 2.0) + bc_params(0.18, 0.0, 2000.0, 2.0)
    p.material_params = np.array(mats, float)
    p.rho = (1000.0, 1460.0)
    p.mu = (1e-3, 5.7e-4)
    p.gravity = (0.0, -9.81, 0.0)
    p.temperature = 273.15 + 20
    # elements and their boundary sub-control-volume faces
    NE = nx * ny
    ex, ey = np.arange(NE) % nx, np.arange(NE) // nx
    v0 = ex + mx * ey
    corners = np.stack([v0, v0 + 1, v0 + mx, v0 + mx + 1], 1)
    p.elem_corner = np.ascontiguousarray(corners.ravel().astype(np.int32))
    volume = np.zeros(N)
    bptr, bcorner, bcenter, bnormal, barea = [0], [], [], [], []
    for e in range(NE):
        lower = np.array([ex[e] * hx, ey[e] * hy])
        upper = np.array([(ex[e] + 1) * hx, (ey[e] + 1) * hy])
        glob = lambda loc: lower + np.asarray(loc) * (upper - lower)
        cg = [glob((c & 1, (c >> 1) & 1)) for c in range(4)]
        edge = [glob(FACE_CENTER[f]) for f in range(4)]
        mid = glob((0.5, 0.5))
        scv = (_quad_area(cg[0], edge[2], mid, edge[0]), _quad_area(cg[1], edge[1], mid, edge[2]),
               _quad_area(cg[2], edge[0], mid, edge[3]), _quad_area(cg[3], edge[3], mid, edge[1]))
        for c in range(4):
            volume[corners[e, c]] += scv[c]
        for f in range(4):
            on = (f == 0 and ex[e] == 0) or (f == 1 and ex[e] == nx - 1) or \
                 (f == 2 and ey[e] == 0) or (f == 3 and ey[e] == ny - 1)
            if not on:
                continue
            length = hy if f < 2 else hx
            for c in FACE_CORNERS[f]:
                loc = (np.array([c & 1, (c >> 1) & 1], float) + np.array(FACE_CENTER[f])) * 0.5
                ip = glob(loc)
                bcorner.append(c)
                bcenter.append((ip[0], ip[1], 0.0))
                bnormal.append((FACE_NORMAL[f][0], FACE_NORMAL[f][1], 0.0))
                barea.append(0.5 * length)
        bptr.append(len(bcorner))
    p.volume = volume
    p.conn_ptr = np.zeros(N + 1, np.int32)
    p.conn_nbr = np.zeros(0, np.int32)
    p.conn_dir = np.zeros(0, np.int32)
    p.conn_normal = np.zeros(0)
    p.conn_center = np.zeros(0)
    p.conn_area = np.zeros(0)
    p.bface_ptr = np.array(bptr, np.int32)
    p.bface_corner = np.array(bcorner, np.int32)
    bcenter = np.array(bcenter)
    p.bface_center = np.ascontiguousarray(bcenter.ravel())
    p.bface_normal = np.ascontiguousarray(np.array(bnormal).ravel())
    p.bface_area = np.array(barea)
    btype, bval = _lens_boundary(bcenter, lx, ly, 1, p.rho[0], -9.81)
    p.bface_type = btype
    p.bface_value = np.ascontiguousarray(bval.ravel())
    p.p1_gradients = 1 if p1 else 0
    p.constraint = np.full(N, -1, np.int32)
    p.init_pv = _lens_initial(pos, ly, 1, p.rho[0], -9.81)
    p.init_meaning = np.zeros(N, np.int32)
    p.info = dict(name="lens-vcfv", nx=nx, ny=ny, nz=1, dim=2, flux="darcy", disc="vcfv",
                  gradients="p1" if p1 else "two-point")
    return p


def blackoil_vcfv(nx=40, ny=20, cell=(10.0, 5.0), sigma=1.0, seed=12345, corey_n=2.0, p_res=330e5,
                  with_wells=True, pvt_rows=10):
    """The black-oil benchmark on a vertex-centred 2D vertical section (the
    reference's reservoir_blackoil_vcfv configuration has a 2D grid,
    reservoirproblem.hh:78): (nx+1) x (ny+1) vertices, gravity along y,
    lognormal permeability (vertical one tenth) and uniform porosity per
    vertex, the PVT tables and Corey relperms of ``blackoil``, no-flow
    boundaries, an injector at vertex (0, 0) and a producer at (nx, ny) as
    constraint vertices."""
    hx, hy = cell
    mx, my = nx + 1, ny + 1
    N = mx * my
    vi = np.arange(N)
    pos = np.zeros((N, 3))
    pos[:, 0] = (vi % mx) * hx
    pos[:, 1] = (vi // mx) * hy
    p = ProblemData(capi.MODEL_BLACKOIL_3P)
    p.center = np.ascontiguousarray(pos.ravel())
    rng = np.random.Generator(np.random.Philox(seed))
    z = rng.standard_normal(N)
    kx = np.exp(math.log(1e-13) + sigma * z)
    p.perm = np.ascontiguousarray(np.stack([kx, 0.1 * kx, np.zeros(N)], 1).ravel())
    rng2 = np.random.Generator(np.random.Philox(seed + 1))
    p.porosity = rng2.uniform(0.15, 0.30, N)
    p.material = np.zeros(N, np.int32)
    p.material_params = np.array([capi.LAW_COREY3P, 0, 0, 0, corey_n, 0, 0, 0], float)
    p.gravity = (0.0, -9.81, 0.0)
    pvt = blackoil_pvt(pvt_rows)
    p.pvt_arrays = pvt
    NE = nx * ny
    ex, ey = np.arange(NE) % nx, np.arange(NE) // nx
    v0 = ex + mx * ey
    corners = np.stack([v0, v0 + 1, v0 + mx, v0 + mx + 1], 1)
    p.elem_corner = np.ascontiguousarray(corners.ravel().astype(np.int32))
    volume = np.zeros(N)
    for c in range(4):
        np.add.at(volume, corners[:, c], hx * hy / 4)
    p.volume = volume
    bptr, bcorner, bcenter, bnormal, barea = [0], [], [], [], []
    for e in range(NE):
        lower = np.array([ex[e] * hx, ey[e] * hy])
        for f in range(4):
            on = (f == 0 and ex[e] == 0) or (f == 1 and ex[e] == nx - 1) or \
                 (f == 2 and ey[e] == 0) or (f == 3 and ey[e] == ny - 1)
            if not on:
                continue
            length = hy if f < 2 else hx
            for c in FACE_CORNERS[f]:
                loc = (np.array([c & 1, (c >> 1) & 1], float) + np.array(FACE_CENTER[f])) * 0.5
                ip = lower + loc * np.array([hx, hy])
                bcorner.append(c)
                bcenter.append((ip[0], ip[1], 0.0))
                bnormal.append((FACE_NORMAL[f][0], FACE_NORMAL[f][1], 0.0))
                barea.append(0.5 * length)
        bptr.append(len(bcorner))
    p.conn_ptr = np.zeros(N + 1, np.int32)
    p.conn_nbr = np.zeros(0, np.int32)
    p.conn_dir = np.zeros(0, np.int32)
    p.conn_normal = np.zeros(0)
    p.conn_center = np.zeros(0)
    p.conn_area = np.zeros(0)
    p.bface_ptr = np.array(bptr, np.int32)
    p.bface_corner = np.array(bcorner, np.int32)
    p.bface_center = np.ascontiguousarray(np.array(bcenter).ravel())
    p.bface_normal = np.ascontiguousarray(np.array(bnormal).ravel())
    p.bface_area = np.array(barea)
    p.bface_type = np.zeros(len(barea), np.int32)
    p.bface_value = np.zeros(4 * len(barea))
    p.p1_gradients = 1
    rs0 = 0.95 * rs_sat(pvt, p_res)
    p.init_pv = np.ascontiguousarray(np.stack([np.zeros(N), np.full(N, p_res), np.full(N, rs0)], 1).ravel())
    p.init_meaning = np.full(N, capi.GAS_RS, np.int32)
    cons = np.full(N, -1, np.int32)
    if with_wells:
        cons[0] = 0
        cons[N - 1] = 1
        p.constraint_pv = np.array([1.0, 1.5 * p_res, 0.0, 0.0, p_res / 1.5, rs0], float)
        p.constraint_meaning = np.array([capi.GAS_SG, capi.GAS_RS], np.int32)
    p.constraint = cons
    p.info = dict(name="blackoil-vcfv", nx=nx, ny=ny, nz=1, dim=2, sigma=sigma, seed=seed, disc="vcfv")
    return p


def _interp(table, x):
    xs = np.array([t[0] for t in table], float)
    ys = np.array([t[1] for t in table], float)
    return np.interp(x, xs, ys)


def blackoil_pvt(rows=10):
    """Reference PVT (reservoirproblem.hh:223-327) with the live-oil table
    resampled to ``rows`` equally spaced pressures in [1.01353e5, 3.45751e7]."""
    p = np.linspace(101353.0, 3.45751e7, rows)
    gas_p = np.array([t[0] for t in REF_BG], float)
    return dict(
        rho_ref=(786.0, 1037.0, 0.97),
        oil_p=p, oil_rs=_interp(REF_RS, p), oil_bo=_interp(REF_BO, p), oil_mu=_interp(REF_MUO, p),
        oil_comp=1.595e-10,
        gas_p=gas_p, gas_bg=np.array([t[1] for t in REF_BG], float),
        gas_mu=np.array([t[1] for t in REF_MUG], float),
        water_p_ref=1.01325e5, water_bw_ref=1.0, water_comp=1.450377e-10, water_mu=9.6e-4,
    )


def rs_sat(pvt, pressure):
    """Saturated R_s by the same piecewise-linear rule the kernels use."""
    x, y = pvt["oil_p"], pvt["oil_rs"]
    n = len(x)
    if pressure <= x[0]:
        i = 0
    elif pressure >= x[-1]:
        i = n - 2
    else:
        i = int(np.searchsorted(x, pressure, side="right") - 1)
    s = (y[i + 1] - y[i]) / (x[i + 1] - x[i])
    return y[i] + s * (pressure - x[i])


def blackoil(nx=100, ny=100, nz=20, cell=(10.0, 10.0, 5.0), sigma=1.0, seed=12345,
             corey_n=2.0, p_res=330e5, with_wells=True, pvt_rows=10):
    """Three-phase black-oil benchmark grid (reservoir problem, synthetic)."""
    lx, ly, lz = nx * cell[0], ny * cell[1], nz * cell[2]
    g = structured_grid(nx, ny, nz, lx, ly, lz, 3)
    p = ProblemData(capi.MODEL_BLACKOIL_3P)
    _fill_grid(p, g)
    N = g["N"]
    rng = np.random.Generator(np.random.Philox(seed))
    z = rng.standard_normal(N)
    kx = np.exp(math.log(1e-13) + sigma * z)
    perm = np.stack([kx, kx, 0.1 * kx], 1)
    p.perm = np.ascontiguousarray(perm.ravel())
    rng2 = np.random.Generator(np.random.Philox(seed + 1))
    p.porosity = rng2.uniform(0.15, 0.30, N)
    p.material = np.zeros(N, np.int32)
    p.material_params = np.array([capi.LAW_COREY3P, 0, 0, 0, corey_n, 0, 0, 0], float)
    p.gravity = (0.0, 0.0, -9.81)
    pvt = blackoil_pvt(pvt_rows)
    p.pvt_arrays = pvt
    nb = len(g["bface_area"])
    p.bface_type = np.zeros(nb, np.int32)
    p.bface_value = np.zeros(4 * nb)
    rs0 = 0.95 * rs_sat(pvt, p_res)
    p.init_pv = np.ascontiguousarray(np.stack([np.zeros(N), np.full(N, p_res), np.full(N, rs0)], 1).ravel())
    p.init_meaning = np.full(N, capi.GAS_RS, np.int32)
    cons = np.full(N, -1, np.int32)
    if with_wells:
        idx = np.arange(N)
        i = idx % nx
        j = (idx // nx) % ny
        inj = (i == 0) & (j == 0)
        prod = (i == nx - 1) & (j == ny - 1)
        cons[inj] = 0
        cons[prod] = 1
        p.constraint_pv = np.array([1.0, 1.5 * p_res, 0.0, 0.0, p_res / 1.5, rs0], float)
        p.constraint_meaning = np.array([capi.GAS_SG, capi.GAS_RS], np.int32)
    p.constraint = cons
    p.info = dict(name="blackoil", nx=nx, ny=ny, nz=nz, dim=3, sigma=sigma, seed=seed)
    return p


def ensemble_member(n_target, seed, sigma):
    """3D two-phase lens-like realisation with about n_target cells: VG
    background material, lognormal permeability, DNAPL inlet on the top
    centre patch and hydrostatic free-flow sides (lensproblem.hh:468-537)."""
    nz = max(2, int(round(n_target ** (1.0 / 3.0))))
    nxy = max(2, int(round(math.sqrt(n_target / nz))))
    nx = ny = nxy
    lx, ly, lz = 6.0, 6.0, 4.0
    g = structured_grid(nx, ny, nz, lx, ly, lz, 3)
    p = ProblemData(capi.MODEL_IMMISCIBLE_2P)
    _fill_grid(p, g)
    N = g["N"]
    rng = np.random.Generator(np.random.Philox(seed))
    kx = np.exp(math.log(4.6e-10) + sigma * rng.standard_normal(N))
    p.perm = np.ascontiguousarray(np.stack([kx, kx, kx], 1).ravel())
    p.porosity = np.full(N, 0.4)
    p.material = np.zeros(N, np.int32)
    p.material_params = np.array(vg_params(0.05, 0.0, 0.0037, 4.7), float)
    p.rho = (1000.0, 1460.0)
    p.mu = (1e-3, 5.7e-4)
    p.gravity = (0.0, 0.0, -9.81)
    eps = 3e-6
    bc = g["bface_center"]
    nb = len(bc)
    btype = np.zeros(nb, np.int32)
    bval = np.zeros((nb, 4))
    on_left = bc[:, 0] < eps
    on_right = bc[:, 0] > lx - eps
    on_top = bc[:, 2] > lz - eps
    depth = lz - bc[:, 2]
    free = on_left | on_right
    pw = np.where(on_left, 1e5 - (1 + 1.5 / lz) * 1000.0 * -9.81 * depth, 1e5 - 1000.0 * -9.81 * depth)
    btype[free] = capi.BC_FREEFLOW
    bval[free, 0] = pw[free]
    bval[free, 1] = 1.0
    inlet = on_top & ~free & (np.abs(bc[:, 0] - lx / 2) < lx / 6) & (np.abs(bc[:, 1] - ly / 2) < ly / 6)
    btype[inlet] = capi.BC_MASSRATE
    bval[inlet, 1] = -0.04
    p.bface_type = btype
    p.bface_value = np.ascontiguousarray(bval.ravel())
    p.constraint = np.full(N, -1, np.int32)
    dep = lz - g["center"][:, 2]
    pw0 = 1e5 - 1000.0 * -9.81 * dep
    p.init_pv = np.ascontiguousarray(np.stack([pw0, np.ones(N)], 1).ravel())
    p.init_meaning = np.zeros(N, np.int32)
    p.info = dict(name="ensemble", nx=nx, ny=ny, nz=nz, dim=3, sigma=sigma, seed=seed)
    return p


def tiny_lens(nx, ny):
    """Small lens-like grids for golden fixtures (same physics, scaled box)."""
    return lens(nx=nx, ny=ny)
