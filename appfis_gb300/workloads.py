"""Seeded synthetic inputs of the five benchmark workloads.

Every random stream is splitmix64 over the element index (counter-based, so any slice can be
regenerated independently): z = seed + (i+1)*0x9E3779B97F4A7C15, two xor-shift-multiply
rounds, U[0,1) = (z >> 11) * 2^-53.  The same generator feeds the GPU path, the oracle and
the CPU baseline, so all three see identical inputs.

Workloads (interior sizes; the reference pads each axis with 2*ghost cells):
  heat2d  1024^2 FP32, U[0,1) interior, Dirichlet UP face (j=0 ghost row) = 1.0, others 0, r=0.2
  gol     16384^2 u8 cells, Bernoulli(0.3), periodic
  himeno  257x257x513 (x, y, z), p = (k/(kmax-1))^2 along z, a0=a1=a2=1, a3=1/6, b*=0, c*=1,
          bnd=1, wrk1=0, omega=0.8, zero ghost ring
  fdtd    512^3 U[-1,1] interior, zero ghost halo of width 4
  triton  32 domains with sides log-uniform in [512, 3072], fractal DEM (spectral exponent
          -2.5, relief 0-50 m), dx=10 m, 1 m of water in a random disc of 5% of the area
"""
import math

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_CHUNK = 1 << 22


def splitmix64(seed, n, start=0):
    """n raw 64-bit outputs of stream `seed`, elements start..start+n-1."""
    out = np.empty(n, dtype=np.uint64)
    s = np.uint64(seed & 0xFFFFFFFFFFFFFFFF)
    with np.errstate(over="ignore"):
        for a in range(0, n, _CHUNK):
            b = min(n, a + _CHUNK)
            z = np.arange(start + a + 1, start + b + 1, dtype=np.uint64)
            z *= _GOLDEN
            z += s
            z ^= z >> np.uint64(30)
            z *= _M1
            z ^= z >> np.uint64(27)
            z *= _M2
            z ^= z >> np.uint64(31)
            out[a:b] = z
    return out


def uniform(seed, n, lo=0.0, hi=1.0, dtype=np.float64):
    """n values U[lo, hi) from stream `seed` (computed in double, then cast)."""
    out = np.empty(n, dtype=dtype)
    for a in range(0, n, _CHUNK):
        b = min(n, a + _CHUNK)
        u = (splitmix64(seed, b - a, start=a) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
        out[a:b] = lo + u * (hi - lo)
    return out


def bernoulli_u8(seed, n, p):
    """n cells, 1 with probability p: U[0,1) < p decided on the 53-bit integer."""
    thr = np.uint64(int(p * 9007199254740992.0))
    out = np.empty(n, dtype=np.uint8)
    for a in range(0, n, _CHUNK):
        b = min(n, a + _CHUNK)
        out[a:b] = (splitmix64(seed, b - a, start=a) >> np.uint64(11)) < thr
    return out


# ------------------------------------------------------------------------------------ heat2d
HEAT2D = dict(nx=1024, ny=1024, iters=1000, r=0.2, top=1.0, seed=42)


def heat2d_padded(nx=1024, ny=1024, top=1.0, seed=42, dtype=np.float32):
    """(ny+2, nx+2) field: U[0,1) interior, ghost row j=0 (UP face) = top, other faces 0."""
    f = np.zeros((ny + 2, nx + 2), dtype=dtype)
    f[1:-1, 1:-1] = uniform(seed, nx * ny).reshape(ny, nx).astype(dtype)
    f[0, :] = top
    return f


# ------------------------------------------------------------------------------------ gol
GOL = dict(nx=16384, ny=16384, gens=2000, p=0.3, seed=42)


def gol_cells(nx=16384, ny=16384, p=0.3, seed=42):
    return bernoulli_u8(seed, nx * ny, p).reshape(ny, nx)


# ------------------------------------------------------------------------------------ himeno
HIMENO = dict(nx=257, ny=257, nz=513, iters=400, omega=0.8)


def himeno_coef(nx, ny, nz, dtype=np.float32, seed=None):
    """12 padded coefficient fields a0 a1 a2 a3 b0 b1 b2 c0 c1 c2 bnd wrk1.  seed=None gives the
    benchmark constants (filled over the whole padded field, as Array::FillData does); a seed
    gives random fields (used by parity tests so every term is exercised)."""
    shape = (12, nz + 2, ny + 2, nx + 2)
    if seed is not None:
        c = uniform(seed, int(np.prod(shape)), 0.0, 1.0).reshape(shape).astype(dtype)
        c[3] *= 0.15  # keep the iteration contractive-ish
        c[4:7] -= 0.5
        c[4:7] *= 0.2
        c[11] -= 0.5
        c[11] *= 0.01
        return c
    c = np.empty(shape, dtype=dtype)
    for k, v in enumerate([1.0, 1.0, 1.0, 1.0 / 6.0, 0.0, 0.0, 0.0, 1.0, 1.0, 1.0, 1.0, 0.0]):
        c[k] = v
    return c


def himeno_p(nx, ny, nz, dtype=np.float32):
    """padded p: (k/(kmax-1))^2 along z over the interior, zero ghost ring."""
    p = np.zeros((nz + 2, ny + 2, nx + 2), dtype=dtype)
    k = np.arange(nz, dtype=np.float64)
    den = max(nz - 1, 1)
    prof = (k / den) ** 2 if dtype == np.float64 else (k.astype(np.float32) / np.float32(den)) ** 2
    p[1:-1, 1:-1, 1:-1] = prof.astype(dtype)[:, None, None]
    return p


# ------------------------------------------------------------------------------------ fdtd
FDTD = dict(nx=512, ny=512, nz=512, iters=200, seed=42, nu=0.1,
            c=(-2.8472, 1.6, -0.2, 0.0254, -0.0018))


def fdtd_weights(c=FDTD["c"], nu=FDTD["nu"]):
    """u <- u + nu * L8(u), L8 = per-axis 8th-order second difference with c0..c4, folded into
    the centre weight 1 + 3*nu*c0 and ring weights nu*c_a (a = 1..4)."""
    return (1.0 + 3.0 * nu * c[0], nu * c[1], nu * c[2], nu * c[3], nu * c[4])


def fdtd_padded(nx=512, ny=512, nz=512, seed=42, dtype=np.float32):
    f = np.zeros((nz + 8, ny + 8, nx + 8), dtype=dtype)
    f[4:-4, 4:-4, 4:-4] = uniform(seed, nx * ny * nz, -1.0, 1.0).reshape(nz, ny, nx).astype(dtype)
    return f


# ------------------------------------------------------------------------------------ triton
TRITON = dict(n_domains=32, side_lo=512, side_hi=3072, dx=10.0, relief=50.0, beta=-2.5, courant=0.5,
              manning=0.035, hextra=1e-3, t_end=600.0, time_step=1.0, h0=1.0, disc_area=0.05, seed=42)


def triton_sizes(n=32, lo=512, hi=3072, seed=42):
    """(ny, nx) per domain, each side log-uniform in [lo, hi]."""
    u = uniform(seed + 7, 2 * n).reshape(n, 2)
    sides = np.rint(lo * np.exp(u * math.log(hi / lo))).astype(np.int64)
    return [(int(a), int(b)) for a, b in sides]


def fractal_dem(ny, nx, seed, beta=-2.5, relief=50.0):
    """Spectral synthesis: white noise shaped to power ~ |k|^beta, scaled to [0, relief] m."""
    noise = uniform(seed, ny * nx, -1.0, 1.0).reshape(ny, nx)
    spec = np.fft.rfft2(noise)
    ky = np.fft.fftfreq(ny)[:, None]
    kx = np.fft.rfftfreq(nx)[None, :]
    k = np.sqrt(kx * kx + ky * ky)
    k[0, 0] = 1.0
    spec *= k ** (beta / 2.0)
    spec[0, 0] = 0.0
    z = np.fft.irfft2(spec, s=(ny, nx))
    z -= z.min()
    z *= relief / max(z.max(), 1e-30)
    return z


def water_disc(ny, nx, seed, h0=1.0, area=0.05):
    """h0 metres inside a disc covering `area` of the domain, centred at a random point."""
    r = math.sqrt(area * nx * ny / math.pi)
    u = uniform(seed + 1, 2)
    cx = r + u[0] * max(nx - 2 * r, 0.0)
    cy = r + u[1] * max(ny - 2 * r, 0.0)
    y, x = np.mgrid[0:ny, 0:nx]
    return np.where((x + 0.5 - cx) ** 2 + (y + 0.5 - cy) ** 2 <= r * r, h0, 0.0)


def triton_domain(ny, nx, seed, beta=-2.5, relief=50.0, h0=1.0, area=0.05):
    return fractal_dem(ny, nx, seed, beta, relief), water_disc(ny, nx, seed, h0, area)


def triton_batch(n=32, lo=512, hi=3072, seed=42, **kw):
    """List of (dem, h) FP64 interiors for the batched workload."""
    return [triton_domain(ny, nx, seed + 1000 * (d + 1), **kw) for d, (ny, nx) in enumerate(triton_sizes(n, lo, hi, seed))]


def write_triton_case(d, nx, ny, seed, duration):
    """The Triton application's input files for one synthetic domain, in directory d: case.cfg
    (key=value), dem.asc (ASCII grid with its 6-line header, dx = 10 m), h.asc (initial depth),
    hydro.txt (a point-source hydrograph) and src.txt (the source at the domain centre), the
    formats the application's readers take (Triton/src/config_utils.hpp, triton_appfis.hpp,
    inflow.hpp).  Values are printed with 6 decimals."""
    import os

    dem, h = triton_domain(ny, nx, seed)

    def grid(path, a, header=""):
        with open(path, "w") as f:
            f.write(header)
            np.savetxt(f, a, fmt="%.6f", delimiter=" ")

    grid(os.path.join(d, "dem.asc"), dem,
         "ncols %d\nnrows %d\nxllcorner 0.0\nyllcorner 0.0\ncellsize 10.0\nNODATA_value -9999\n" % (nx, ny))
    grid(os.path.join(d, "h.asc"), h)
    with open(os.path.join(d, "hydro.txt"), "w") as f:
        f.write("% time (hr), flow (m3/s)\n0, 0\n0.01, 8.0\n0.03, 3.0\n1.0, 0.0\n")
    with open(os.path.join(d, "src.txt"), "w") as f:
        f.write("%% x, y\n%.1f, %.1f\n" % (10.0 * (nx // 2) - 5.0, 10.0 * (ny // 2) - 5.0))
    cfg = dict(dem_filename="dem.asc", h_infile="h.asc", hydrograph_filename="hydro.txt", src_loc_file="src.txt",
               num_sources=1, const_mann=0.035, time_step=1.0, time_increment_fixed=0, time_series_flag=0, courant=0.5,
               hextra=0.001, gpu_direct_flag=0, num_runoffs=0, num_extbc=0, print_option="h", input_format="ASC",
               output_format="ASC", output_option="SEQ", sim_start_time=0, sim_duration=duration, print_interval=60)
    with open(os.path.join(d, "case.cfg"), "w") as f:
        f.write("".join("%s=%s\n" % kv for kv in cfg.items()))

