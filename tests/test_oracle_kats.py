"""CPU: known-answer tests of the FP64 oracle against independent numpy
statements of the same mathematics (the oracle is also pinned to the
reference's own CPU build through the golden fixtures; these pin it a second
way, without the reference).

* one point's Fresnel CGH is the analytic chirp
  exp(i pi ((p w - x)^2 + (p h - y)^2) / (lambda z)) (golcgh.h:47-88);
* one point's exact CGH is a exp(i (k r + phi)) / r;
* ASM (golprop.h:507-534) equals crop(IFFT(H . FFT(pad u))) with numpy's FFT,
  the field padded into the centre of a 2ny x 2nx grid (golutils.h:197-199),
  H = exp(2 pi i z sqrt(1/lambda^2 - fx^2 - fy^2)) on numpy's frequency grid
  and the crop [ny/2, 3ny/2) x [nx/2, 3nx/2) (golutils.h:255-257);
* ASM by z then by -z returns a field that stays inside the window."""
import numpy as np

import oracle as O


def test_single_point_fresnel_cgh_is_the_analytic_chirp():
    ny, nx, p, lam = 24, 40, 8e-6, 532e-9
    x0, y0, z0 = 17.3 * p, 9.8 * p, 0.1
    U = O.cgh_fresnel(np.array([[x0, y0, z0]]), ny, nx, p, p, lam)
    h, w = np.mgrid[0:ny, 0:nx]
    ref = np.exp(1j * np.pi * ((p * w - x0) ** 2 + (p * h - y0) ** 2) / (lam * z0))
    assert np.abs(U - ref).max() < 1e-12


def test_single_point_exact_cgh_is_the_spherical_wave():
    ny, nx, p, lam = 20, 28, 8e-6, 633e-9
    x0, y0, z0, a, phi = 11.5 * p, 6.25 * p, 0.05, 0.7, 1.3
    U = O.cgh_exact(np.array([[x0, y0, z0]]), ny, nx, p, p, lam, amp=np.array([a]), phase0=np.array([phi]))
    h, w = np.mgrid[0:ny, 0:nx]
    r = np.sqrt((p * w - x0) ** 2 + (p * h - y0) ** 2 + z0 ** 2)
    ref = a * np.exp(1j * (2 * np.pi / lam * r + phi)) / r
    assert np.abs(U - ref).max() / np.abs(ref).max() < 1e-9


def numpy_asm(u, dy, dx, lam, z):
    ny, nx = u.shape
    pad = np.zeros((2 * ny, 2 * nx), np.complex128)
    pad[ny // 2:ny // 2 + ny, nx // 2:nx // 2 + nx] = u
    fy = np.fft.fftfreq(2 * ny, dy)[:, None]
    fx = np.fft.fftfreq(2 * nx, dx)[None, :]
    H = np.exp(2j * np.pi * z * np.sqrt(1.0 / lam ** 2 - fx ** 2 - fy ** 2))
    out = np.fft.ifft2(np.fft.fft2(pad) * H)
    return out[ny // 2:ny // 2 + ny, nx // 2:nx // 2 + nx]


def test_asm_equals_the_numpy_statement():
    rng = np.random.default_rng(5)
    for (ny, nx), (dy, dx), lam, z in [((64, 96), (8e-6, 8e-6), 532e-9, 0.02),
                                        ((48, 32), (6e-6, 4e-6), 633e-9, -0.01),
                                        ((128, 128), (8e-6, 8e-6), 450e-9, 0.05)]:
        u = (rng.random((ny, nx)) < 0.5) * np.exp(2j * np.pi * rng.random((ny, nx)))
        got = O.asm_prop(u, dy, dx, lam, z)
        ref = numpy_asm(u, dy, dx, lam, z)
        # the phase 2 pi z / lambda ~ 1e5 rad rounds differently in the two
        # evaluation orders (~1e-11); a grid or shift convention error is O(1)
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-9, (ny, nx, z)


def test_asm_of_a_delta_is_the_cropped_impulse_response():
    # a delta at the window centre: the output is the centred crop of IFFT(H)
    # rolled to the delta's position in the padded grid
    ny, nx, dy, dx, lam, z = 32, 48, 8e-6, 8e-6, 532e-9, 0.004
    u = np.zeros((ny, nx), np.complex128)
    u[ny // 2, nx // 2] = 1.0
    fy = np.fft.fftfreq(2 * ny, dy)[:, None]
    fx = np.fft.fftfreq(2 * nx, dx)[None, :]
    h = np.fft.ifft2(np.exp(2j * np.pi * z * np.sqrt(1.0 / lam ** 2 - fx ** 2 - fy ** 2)))
    h = np.roll(h, (ny, nx), axis=(0, 1))  # delta at padded (ny, nx)
    ref = h[ny // 2:ny // 2 + ny, nx // 2:nx // 2 + nx]
    got = O.asm_prop(u, dy, dx, lam, z)
    assert np.abs(got - ref).max() < 1e-12


def test_asm_forward_then_back_is_the_identity_inside_the_window():
    ny, nx, p, lam, z = 128, 128, 8e-6, 532e-9, 0.002
    h, w = np.mgrid[0:ny, 0:nx]
    # a smooth beam well inside the window: nothing diffracts out of it
    u = np.exp(-(((h - ny / 2) / 10.0) ** 2 + ((w - nx / 2) / 12.0) ** 2)) * np.exp(0.3j * (h - w) / ny)
    back = O.asm_prop(O.asm_prop(u, p, p, lam, z), p, p, lam, -z)
    assert np.linalg.norm(back - u) / np.linalg.norm(u) < 1e-9
