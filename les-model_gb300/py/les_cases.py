"""Workload definitions: grids, obstacles and seeded initial fields.

The five workloads are synthetic stand-ins with the shapes of the les-model
benchmark configurations (no dataset is involved):

  small     64x32x32, h = 1/32, cube obstacle [16,24)x[12,20)x[12,20)
  large     256x128x128, h = 1/128, the same obstacle scaled 4x
  xlarge    512x256x256, h = 1/256, scaled 8x
  adjoint   128x64x64, h = 1/64, centred cube (the small obstacle scaled 2x)
  batch     ragged grids with dims in {32,48,64,80,96}, cube side
            floor(min(dims)/4) at a seeded position

Initial state: u = 1 + U(-a, a), v = w = U(-a, a) (a = 0.01; 0.02 for the
batch), p = 0, drawn from numpy's PCG64 with the given seed in the order u, v,
w, then apply_velocity_BCs.  The pressure matrix is assembled before the mask
is defined, as src/main.cpp:66-81 does.
"""
import numpy as np

CONFIGS = {
    "small": dict(shape=(64, 32, 32), h=1.0 / 32, box=(16, 24, 12, 20, 12, 20), noise=0.01),
    "large": dict(shape=(256, 128, 128), h=1.0 / 128, box=(64, 96, 48, 80, 48, 80), noise=0.01),
    "xlarge": dict(shape=(512, 256, 256), h=1.0 / 256, box=(128, 192, 96, 160, 96, 160), noise=0.01),
    "adjoint": dict(shape=(128, 64, 64), h=1.0 / 64, box=(32, 48, 24, 40, 24, 40), noise=0.01),
}

# physics of the configurations
NU, RHO, CS = 1e-5, 1.2, 0.17
CFL_CONV, CFL_VISC, DT_MAX = 0.3, 0.2, 1e-4


def box_mask(shape, box):
    nx, ny, nz = shape
    s = np.zeros(shape, np.uint8)
    i0, i1, j0, j1, k0, k1 = box
    s[i0:i1, j0:j1, k0:k1] = 1
    return s.reshape(-1)


def init_fields(shape, noise, seed):
    n = shape[0] * shape[1] * shape[2]
    rng = np.random.default_rng(seed)
    u = 1.0 + rng.uniform(-noise, noise, n)
    v = rng.uniform(-noise, noise, n)
    w = rng.uniform(-noise, noise, n)
    z = lambda: np.zeros(n)  # noqa: E731
    return dict(u=u, v=v, w=w, u_new=z(), v_new=z(), w_new=z(), p=z(), p_rhs=z(), nu_t=z())


def velocity_bcs_np(shape, f, solid):
    """apply_velocity_BCs (src/main.cpp:323-410) in numpy, for host-side setup."""
    nx, ny, nz = shape
    s = solid.reshape(shape).astype(bool)
    for key in ("u", "v", "w"):
        a = f[key].reshape(shape)
        inlet = ~s[0]
        a[0][inlet] = 1.0 if key == "u" else 0.0
        a[nx - 1] = a[nx - 2]
        a[:, 0, :] = 0.0
        a[:, ny - 1, :] = 0.0
        a[:, :, 0] = 0.0
        a[:, :, nz - 1] = 0.0
        inner = np.zeros(shape, bool)
        inner[1:-1, 1:-1, 1:-1] = s[1:-1, 1:-1, 1:-1]
        a[inner] = 0.0


def case(name, seed=1234):
    c = CONFIGS[name]
    shape = c["shape"]
    solid = box_mask(shape, c["box"])
    f = init_fields(shape, c["noise"], seed)
    velocity_bcs_np(shape, f, solid)
    return shape, c["h"], solid, f


def batch_cases(count=64, seed=7, noise=0.02):
    """Ragged ensemble: per-case dims, obstacle and Cs drawn from the seed."""
    rng = np.random.default_rng(seed)
    dims = (32, 48, 64, 80, 96)
    out = []
    for q in range(count):
        shape = tuple(int(rng.choice(dims)) for _ in range(3))
        side = min(shape) // 4
        pos = [int(rng.integers(1, shape[a] - side - 1)) for a in range(3)]
        box = (pos[0], pos[0] + side, pos[1], pos[1] + side, pos[2], pos[2] + side)
        cs = float(rng.uniform(0.1, 0.2))
        out.append(dict(shape=shape, h=1.0 / 32, box=box, cs=cs, seed=int(rng.integers(1 << 31)),
                        noise=noise))
    return out
