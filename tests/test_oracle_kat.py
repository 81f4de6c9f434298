"""The oracle against the reference's own self-contained tests.

Each test restates a testset of SPHtoGrid.jl's test/runtests.jl (line numbers
cited) on the C oracle; a second pure-Python restatement cross-checks the C
oracle bit for bit on small random cases.
"""
import math

import numpy as np
import pytest

KERNELS = ["cubic", "quintic", "wendlandc4", "wendlandc6", "wendlandc8"]


def test_mapping_parameters_errors(oracle):
    # runtests.jl:38-58
    with pytest.raises(oracle.OracleError, match="Giving a center position requires extent"):
        oracle.mapping_parameters()
    with pytest.raises(oracle.OracleError, match="Please specify pixelSideLength or number of pixels!"):
        oracle.mapping_parameters(center=[0.0, 0.0, 0.0], x_lim=[-1.0, 1.0], y_lim=[-1.0, 1.0],
                                  z_lim=[-1.0, 1.0])
    p = oracle.mapping_parameters(center=[0.0, 0.0, 0.0], x_lim=[-1.0, 1.0], y_lim=[-1.0, 1.0],
                                  z_lim=[-1.0, 1.0], Npixels=100)
    assert p.Npixels[0] == 100 and p.pixelSideLength == 0.02
    p = oracle.mapping_parameters(center=[0.0, 0.0, 0.0], x_lim=[-1.0, 1.0], y_lim=[-1.0, 1.0],
                                  z_lim=[-1.0, 1.0], pixelSideLength=0.2)
    assert p.Npixels[0] == 10 and p.len2pix == 5.0


def test_filter_particles(oracle):
    # runtests.jl:60-77
    par = oracle.mapping_parameters(center=[3.0, 3.0, 3.0], x_size=6.0, y_size=6.0, z_size=6.0,
                                    Npixels=500)
    x = np.zeros((3, 2), order="F")
    x[:, 0] = [1.0, 1.0, 1.0]
    x[:, 1] = [-5.0, -1.0, 1.0]
    mask = oracle.filter_particles_in_image(x, par)
    assert mask[0] and not mask[1]


def test_filter_is_inclusive(oracle):
    # filter_shift.jl:50: lower <= x <= upper
    par = oracle.mapping_parameters(center=[0.0, 0.0, 0.0], x_size=2.0, y_size=2.0, z_size=2.0,
                                    Npixels=8)
    x = np.array([[1.0, -1.0, np.nextafter(1.0, 2.0), 0.0],
                  [0.0, 1.0, 0.0, np.nan],
                  [-1.0, 0.0, 0.0, 0.0]])
    assert oracle.filter_particles_in_image(x, par).tolist() == [True, True, False, False]


def test_shift_particles(oracle):
    # runtests.jl:79-99
    par = oracle.mapping_parameters(center=[1.0, 1.0, 1.0], x_size=6.0, y_size=6.0, z_size=6.0,
                                    Npixels=500)
    x = np.zeros((3, 2), order="F")
    x[:, 0] = [1.0, 1.0, 1.0]
    x[:, 1] = [-3.0, -1.0, 1.0]
    par2 = oracle.center_particles(x, par)
    np.testing.assert_allclose(x[:, 0], [0.0, 0.0, 0.0])
    np.testing.assert_allclose(x[:, 1], [-4.0, -2.0, 0.0])
    assert list(par.center) == [1.0, 1.0, 1.0]
    assert list(par2.center) == [0.0, 0.0, 0.0]


def test_shift_float32_rounds_in_place(oracle):
    # filter_shift.jl:15: the difference is stored back into the Float32 array
    par = oracle.mapping_parameters(center=[0.1, 0.2, 0.3], x_size=1.0, y_size=1.0, z_size=1.0,
                                    Npixels=16)
    x = np.asfortranarray(np.array([[0.7], [0.11], [1e-3]], dtype=np.float32))
    orig = x.astype(np.float64)
    oracle.center_particles(x, par)
    want = (orig - np.array([[0.1], [0.2], [0.3]])).astype(np.float32)
    assert np.array_equal(x, want)


def test_periodic_shift_quirk(oracle):
    # filter_shift.jl:18-21: |x| > boxsize/2 is shifted by boxsize/2
    par = oracle.mapping_parameters(center=[0.0, 0.0, 0.0], x_size=4.0, y_size=4.0, z_size=4.0,
                                    Npixels=8, boxsize=2.0)
    assert par.periodic
    x = np.array([[1.5], [-1.5], [0.5]])
    oracle.center_particles(x, par)
    assert x[:, 0].tolist() == [0.5, -0.5, 0.5]


@pytest.mark.parametrize("npix", [128])
def test_indices_bijection(oracle, npix):
    # runtests.jl:139-166
    n2 = npix * npix
    seen = np.zeros(n2, dtype=np.int64)
    count = 1
    for i in range(npix):
        for j in range(npix):
            seen[oracle.calculate_index(i, j, npix) - 1] = count
            count += 1
    assert np.array_equal(seen, np.arange(1, n2 + 1))
    n3 = npix ** 3
    seen = np.zeros(n3, dtype=np.int64)
    idx = np.array([oracle.calculate_index(i, j, k, npix, npix)
                    for i in range(npix) for j in range(npix) for k in range(npix)])
    seen[idx - 1] = np.arange(1, n3 + 1)
    assert np.array_equal(seen, np.arange(1, n3 + 1))


def test_mass_conservation_3d(oracle):
    # runtests.jl:324-342 (Cubic, npix=200, r=64, single particle)
    npix, r = 200, 64
    par = oracle.mapping_parameters(x_lim=[-r, r], y_lim=[-r, r], z_lim=[-r, r], Npixels=npix)
    pos = np.array([[0.0101], [-0.001], [0.001]])
    hsml, mass, rho = np.array([5]), np.array([3]), np.ones(1)
    w = np.ones(1) * par.pixelSideLength  # part_weight_physical(N, par, 1)
    img, _ = oracle.sph_mapping(pos, hsml, mass, rho, rho, w, param=par, dimensions=3,
                                kernel="cubic", reduce_image=False)
    vpix = (par.x_lim[1] - par.x_lim[0]) ** 3 / npix ** 3
    assert math.isclose(vpix * img.sum(), 3.0, rel_tol=math.sqrt(np.finfo(float).eps))


def test_particle_not_overlapping_centres_2d(oracle):
    # runtests.jl:718-738 (fallback branch, rtol 1e-10)
    npix, r = 4, 10
    par = oracle.mapping_parameters(x_lim=[-r, r], y_lim=[-r, r], z_lim=[-r, r], Npixels=npix)
    pos = np.array([[0.5], [0.0], [0.0]])
    hsml, mass, rho = np.array([1.0]), np.array([1.0]), np.ones(1)
    w = np.ones(1) * par.pixelSideLength
    img, _ = oracle.sph_mapping(pos, hsml, mass, rho, rho, w, param=par, kernel="cubic",
                                kernel_dim=3, reduce_image=False)
    apix = (par.x_lim[1] - par.x_lim[0]) ** 2 / npix ** 2
    assert math.isclose(apix * img.sum(), 1.0, rel_tol=1e-10)


@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("kdim", [2, 3])
def test_kernel_normalisation(oracle, kernel, kdim):
    """The restated SPHKernels shapes integrate to one over the support and
    vanish at u = 1 (midpoint rule, h = 1)."""
    n = 200000
    u = (np.arange(n) + 0.5) / n
    w = np.array([oracle.kernel_value(kernel, kdim, float(x), 1.0) for x in u[::50]])
    uu = u[::50]
    shell = 2 * np.pi * uu if kdim == 2 else 4 * np.pi * uu ** 2
    integral = (w * shell).sum() * (50.0 / n)
    assert abs(integral - 1.0) < 2e-4
    assert oracle.kernel_value(kernel, kdim, 1.0, 1.0) == 0.0
    assert oracle.kernel_value(kernel, kdim, 0.0, 1.0) > 0.0


def _random_case(rng, n, dims, nq, dtype):
    pos = rng.uniform(-0.55, 0.55, (3, n))
    hsml = np.exp(rng.uniform(np.log(0.01), np.log(0.3), n))
    m = rng.uniform(0.5, 1.5, n) / n
    rho = rng.uniform(0.5, 2.0, n)
    q = rng.uniform(-1.0, 2.0, (nq, n)) if nq > 1 else rng.uniform(0.5, 2.0, n)
    if nq > 1:
        q[:, :3] = 0.0
    else:
        q[:3] = 0.0
    w = rng.uniform(0.5, 2.0, n)
    cast = lambda a: a.astype(dtype)
    return cast(np.asfortranarray(pos)), cast(hsml), cast(m), cast(rho), cast(q), cast(w)


@pytest.mark.parametrize("dims,nq,kernel,dtype,calc_mean", [
    (2, 1, "cubic", np.float64, False),
    (2, 3, "quintic", np.float64, True),
    (2, 2, "wendlandc4", np.float32, False),
    (3, 1, "wendlandc6", np.float64, False),
    (3, 1, "wendlandc8", np.float32, False),
])
def test_c_oracle_matches_python_restatement(oracle, pyoracle, dims, nq, kernel, dtype, calc_mean):
    rng = np.random.default_rng(dims * 10 + nq)
    n = 40 if dims == 3 else 120
    P = 12 if dims == 3 else 24
    pos, hsml, m, rho, q, w = _random_case(rng, n, dims, nq, dtype)
    par = oracle.mapping_parameters(center=[0.0, 0.0, 0.0], x_size=1.0, y_size=1.0, z_size=1.0,
                                    Npixels=P)
    raw = dims == 2
    img, info = oracle.sph_mapping(pos, hsml, m, rho, q, w, param=par, kernel=kernel,
                                   dimensions=dims, return_both_maps=raw, reduce_image=False,
                                   calc_mean=calc_mean)
    # python restatement on the filtered particles
    mask = oracle.filter_particles_in_image(pos, par)
    idx = np.nonzero(mask)[0]
    qq = q.reshape(nq, -1)
    chans, dep = pyoracle.cic_map(dims, [tuple(pos[:, i]) for i in idx], hsml[idx], m[idx],
                                  rho[idx], [tuple(qq[:, i]) for i in idx], w[idx], par.len2pix, P,
                                  kernel, calc_mean=calc_mean and dims == 2)
    assert dep == info["deposits"]
    PD = P ** dims
    if raw:
        for ch in range(nq + 1):
            dense = np.zeros(PD)
            for k, v in chans[ch].items():
                dense[k] = v
            assert np.array_equal(dense, img[:, ch]), f"channel {ch}"
    else:
        q_dense = np.zeros(PD)
        for k, v in chans[0].items():
            q_dense[k] = v
        # 3D with reduce_image = false: W is set to 1 (cic_interpolation.jl:230-232)
        assert np.array_equal(img.reshape(-1, order="F"), q_dense)


def test_threaded_oracle_matches_serial(oracle):
    rng = np.random.default_rng(5)
    pos, hsml, m, rho, q, w = _random_case(rng, 3000, 2, 2, np.float64)
    par = oracle.mapping_parameters(center=[0.0, 0.0, 0.0], x_size=1.0, y_size=1.0, z_size=1.0,
                                    Npixels=48)
    a, ia = oracle.sph_mapping(pos, hsml, m, rho, q, w, param=par, kernel="cubic", nthreads=1)
    b, ib = oracle.sph_mapping(pos, hsml, m, rho, q, w, param=par, kernel="cubic", nthreads=4)
    assert ia["deposits"] == ib["deposits"]
    np.testing.assert_allclose(b, a, rtol=1e-12, atol=1e-14 * np.abs(a).max())


def test_volume_conservation_property_2d(oracle):
    """Sum of the weight image = sum over mapped particles of w m L^3 / rho
    (the closed form of cic_2D.jl:187-199)."""
    rng = np.random.default_rng(11)
    pos, hsml, m, rho, q, w = _random_case(rng, 2000, 2, 1, np.float64)
    par = oracle.mapping_parameters(center=[0.0, 0.0, 0.0], x_size=1.0, y_size=1.0, z_size=1.0,
                                    Npixels=40)
    p0 = pos.copy()
    img, _ = oracle.sph_mapping(pos, hsml, m, rho, q, w, param=par, kernel="wendlandc4",
                                return_both_maps=True)
    mask = oracle.filter_particles_in_image(p0, par) & (q != 0)
    L = par.len2pix
    want = (w * m * L ** 3 / rho)[mask].sum()
    assert math.isclose(img[:, -1].sum(), want, rel_tol=1e-12)


def test_sort_z_selection_quirk(oracle):
    """filter_shift.jl:61-63 indexes the z-sorted permutation with the mask in
    input order; the oracle keeps that selection."""
    par = oracle.mapping_parameters(center=[0.0, 0.0, 0.0], x_size=1.0, y_size=1.0, z_size=1.0,
                                    Npixels=8)
    # A, B inside; C outside in z only.  mask = [T, T, F]; z = [0.3, -0.2, 0.9]
    # reverse(sortperm(z)) = [C, A, B]; indexed by the mask -> [C, A]
    pos = np.array([[0.0, 0.1, 0.2], [0.0, 0.1, -0.1], [0.3, -0.2, 0.9]])
    one = np.ones(3)
    hs = np.full(3, 0.1)
    img_s, _ = oracle.sph_mapping(pos.copy(), hs, one, one, one, one, param=par, kernel="cubic",
                                  sort_z=True, return_both_maps=True)
    pos_ac = pos[:, [0, 2]].copy()
    pos_ac[2, 1] = 0.0  # C moved inside in z: same 2D footprint
    img_ac, _ = oracle.sph_mapping(pos_ac, hs[:2], one[:2], one[:2], one[:2], one[:2], param=par,
                                   kernel="cubic", return_both_maps=True)
    np.testing.assert_allclose(img_s, img_ac, rtol=1e-14, atol=0)
