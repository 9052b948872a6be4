"""Surface and target-layer setup: drop-in for ``src/PYTHON/simple_surfaces.py``.

Same functions, signatures and file formats as the reference
(``gen_normals`` simple_surfaces.py:3-39, ``export_facets`` :65-85,
``export_targets`` :88-107, ``make_surface`` :147-201,
``make_target_array`` :204-254).  ``surface_arrays`` / ``target_arrays``
return the same data as SoA arrays for the file-free path
(``simulate(params, facets, targets)``).
"""
import numpy as np


def gen_normals(params, fzzs):
    """Normals by central differences, tangents by cross products
    (simple_surfaces.py:3-39)."""
    dZdx = np.zeros_like(fzzs)
    dZdy = np.zeros_like(fzzs)
    dZdx[:, 1:-1] = (fzzs[:, 2:] - fzzs[:, :-2]) / (2 * params["fs"])
    dZdy[1:-1, :] = (fzzs[2:, :] - fzzs[:-2, :]) / (2 * params["fs"])
    dZdx[:, 0] = dZdx[:, 1]
    dZdx[:, -1] = dZdx[:, -2]
    dZdy[0, :] = dZdy[1, :]
    dZdy[-1, :] = dZdy[-2, :]
    norms = np.sqrt(dZdx ** 2 + dZdy ** 2 + 1)
    ny, nx = fzzs.shape
    n_hat = np.zeros((ny, nx, 3))
    n_hat[:, :, 0] = -dZdx / norms
    n_hat[:, :, 1] = -dZdy / norms
    n_hat[:, :, 2] = 1 / norms
    ref = np.zeros_like(n_hat)
    ref[:, :, 0] = 1
    parallel_mask = np.abs(n_hat[:, :, 0]) > 0.9
    ref[parallel_mask, :] = [0, 1, 0]
    u_hat = np.cross(ref, n_hat)
    u_hat /= np.linalg.norm(u_hat, axis=2, keepdims=True)
    v_hat = np.cross(n_hat, u_hat)
    return n_hat, u_hat, v_hat


def export_facets(fxs, fys, fzs, fnxs, fnys, fnzs, fuxs, fuys, fuzs, fvxs, fvys, fvzs,
                  filename, obj=None):
    """Facet file ``x,y,z:nx,ny,nz:ux,uy,uz:vx,vy,vz`` with 6 decimals,
    no newline after the last record (simple_surfaces.py:65-76)."""
    n = len(fxs)
    with open(filename, "w") as f:
        for i, (x, y, z, nx, ny, nz, ux, uy, uz, vx, vy, vz) in enumerate(
                zip(fxs, fys, fzs, fnxs, fnys, fnzs, fuxs, fuys, fuzs, fvxs, fvys, fvzs)):
            f.write(f"{x:.6f},{y:.6f},{z:.6f}:{nx:.6f},{ny:.6f},{nz:.6f}:"
                    f"{ux:.6f},{uy:.6f},{uz:.6f}:{vx:.6f},{vy:.6f},{vz:.6f}")
            if i != n - 1:
                f.write("\n")
    print(f"Exported facet data to: {filename}")


def export_targets(fxs, fys, fzs, fnxs, fnys, fnzs, filename, obj=None):
    """Target file ``x,y,z,nx,ny,nz,1`` with 6 decimals (simple_surfaces.py:88-107)."""
    n = len(fxs)
    with open(filename, "w") as f:
        for i, (x, y, z, nx, ny, nz) in enumerate(zip(fxs, fys, fzs, fnxs, fnys, fnzs)):
            f.write(f"{x:.6f},{y:.6f},{z:.6f},{nx:.6f},{ny:.6f},{nz:.6f},1")
            if i != n - 1:
                f.write("\n")


def gen_flat(params, fzzs):
    return np.zeros_like(fzzs)


def gen_concave(params, fxxs, fyys, fzzs):
    R = params["sz"]
    r2 = fxxs ** 2 + fyys ** 2
    return R - np.sqrt(np.maximum(0, R ** 2 - r2))


def gen_convex(params, fxxs, fyys, fzzs):
    R = params["sz"]
    r2 = fxxs ** 2 + fyys ** 2
    return np.sqrt(np.maximum(0, R ** 2 - r2)) - R


def calc_fresnel(params, debug=False):
    Fr = np.sqrt((params["sz"] + params["lam"] / 4) ** 2 - params["sz"] ** 2)
    if debug:
        print(f"Calculated fresnel zone radius as {Fr:.2f} meters")
    return Fr


def calc_fresnel_spherical(params, debug=False):
    h = params["sz"]
    r = params["sz"]
    Fr = np.sqrt((params["lam"] * h * r) / (2 * (h + r)))
    if debug:
        print(f"Calculated fresnel zone radius as {Fr:.2f} meters")
    return Fr


def gen_fresnel(params, fxxs, fyys, fzzs, stype="flat"):
    fxys = np.sqrt(fxxs ** 2 + fyys ** 2)
    if stype == "flat":
        fzzs = gen_flat(params, fzzs)
        Fr = calc_fresnel(params)
    elif stype == "convex":
        fzzs = gen_convex(params, fxxs, fyys, fzzs)
        Fr = calc_fresnel_spherical(params)
    mask = fxys <= Fr
    return fzzs, mask


def _grid(params):
    fxs = np.arange(params["nx"]) * params["fs"] + params["ox"]
    fys = np.arange(params["ny"]) * params["fs"] + params["oy"]
    fxxs, fyys = np.meshgrid(fxs, fys)
    return fxxs, fyys, np.zeros_like(fxxs)


def _soa(fxxs, fyys, fzzs, n_hat, u_hat, v_hat, mask=None):
    cols = [fxxs, fyys, fzzs] + [a[:, :, i] for a in (n_hat, u_hat, v_hat) for i in range(3)]
    soa = np.stack([c.flatten() for c in cols])
    if mask is not None:
        soa = soa[:, mask.flatten()]
    return soa


def surface_arrays(params, stype, heights=None):
    """Facets of ``make_surface`` as a (12, N) SoA array (no file).

    ``heights`` (ny, nx) overrides the named surface type (used by the
    seeded rough-surface generators)."""
    fxxs, fyys, fzzs = _grid(params)
    mask = None
    if heights is not None:
        fzzs = np.asarray(heights, dtype=np.float64)
    elif stype == "flat":
        fzzs = gen_flat(params, fzzs)
    elif stype == "concave":
        fzzs = gen_concave(params, fxxs, fyys, fzzs)
    elif stype == "fresnel":
        fzzs, mask = gen_fresnel(params, fxxs, fyys, fzzs, stype="flat")
    elif stype == "fresnel-convex":
        fzzs, mask = gen_fresnel(params, fxxs, fyys, fzzs, stype="convex")
    else:
        raise ValueError(f"Unknown surface type: {stype}")
    n_hat, u_hat, v_hat = gen_normals(params, fzzs)
    return _soa(fxxs, fyys, fzzs, n_hat, u_hat, v_hat, mask)


def surface_arrays_blocked(params, heights, rows_per_block=256):
    """``surface_arrays(params, "flat", heights)`` for large grids, by blocks
    of rows: the same values bit for bit (``gen_normals`` runs on each block
    with two halo rows on either side, so the grid's edge rows keep its edge
    rule), without the whole-grid (ny, nx, 3) temporaries."""
    z = np.asarray(heights, dtype=np.float64)
    ny, nx = z.shape
    if ny < 3:
        return surface_arrays(params, "flat", heights=z)
    out = np.empty((12, ny * nx))
    xs = np.arange(nx) * params["fs"] + params["ox"]
    ys = np.arange(ny) * params["fs"] + params["oy"]
    for r0 in range(0, ny, rows_per_block):
        r1 = min(ny, r0 + rows_per_block)
        h0, h1 = max(0, r0 - 2), min(ny, r1 + 2)
        n_hat, u_hat, v_hat = gen_normals(params, z[h0:h1])
        a, b = r0 - h0, r0 - h0 + (r1 - r0)
        sl = slice(r0 * nx, r1 * nx)
        out[0, sl] = np.tile(xs, r1 - r0)
        out[1, sl] = np.repeat(ys[r0:r1], nx)
        out[2, sl] = z[r0:r1].ravel()
        for k, arr in enumerate((n_hat, u_hat, v_hat)):
            for i in range(3):
                out[3 + 3 * k + i, sl] = arr[a:b, :, i].ravel()
    return out


def make_surface(params, stype, filename, obj=None):
    """Write a facet file for a named surface (simple_surfaces.py:147-201)."""
    soa = surface_arrays(params, stype)
    export_facets(*soa, filename, obj=obj)


def target_arrays(params, ttype, zoffset=0, heights=None):
    """Targets of ``make_target_array`` as a (7, T) SoA array (ttype column 1)."""
    fxxs, fyys, fzzs = _grid(params)
    if heights is not None:
        fzzs = np.asarray(heights, dtype=np.float64).copy()
    elif ttype == "flat":
        fzzs = gen_flat(params, fzzs)
    fzzs = fzzs + zoffset
    n_hat, u_hat, v_hat = gen_normals(params, fzzs)
    soa = _soa(fxxs, fyys, fzzs, n_hat, u_hat, v_hat)
    return np.concatenate([soa[:6], np.ones((1, soa.shape[1]))], axis=0)


def make_target_array(params, ttype, filename, obj=None, zoffset=0):
    """Write a target-layer file (simple_surfaces.py:204-254)."""
    soa = target_arrays(params, ttype, zoffset=zoffset)
    print(f"Target count: ntargets = {soa.shape[1]}")
    export_targets(*soa[:6], filename, obj=obj)
