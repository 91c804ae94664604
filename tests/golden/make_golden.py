"""Generate the golden fixtures in this folder from the XLuminA reference source.

Run in a container that holds the reference checkout (read-only is fine):

    python tests/golden/make_golden.py /path/to/XLuminA

The reference is pure Python on jax; jax is not installable here, so
``jax_numpy_standin.install()`` first registers a numpy-backed stand-in for the
jax calls the reference makes (float64 / complex128 throughout, as the
reference forces ``jax_enable_x64``).  The reference's own functions then run
unchanged on small seeded inputs and their outputs are written as ``.npz``
fixtures.  The fixtures travel with the repository; the tests never need the
reference checkout.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _save(name, **arrays):
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **{k: np.asarray(v) for k, v in arrays.items()})
    print("wrote", path)


def main(ref_root):
    sys.path.insert(0, HERE)
    import jax_numpy_standin

    jax_numpy_standin.install()
    sys.path.insert(0, ref_root)
    import contextlib
    import io

    from xlumina import loss_functions as lf
    from xlumina import optical_elements as oe
    from xlumina import toolbox as tb
    from xlumina.vectorized_optics import PolarizedLightSource, VectorizedLight
    from xlumina.wave_optics import LightSource, ScalarLight

    quiet = contextlib.redirect_stdout(io.StringIO())
    rng = np.random.default_rng(1234)

    with quiet:
        # 1. scalar RS, square grid, SLM-modulated Gaussian, z > 0 and z < 0.
        x, y = tb.space(150.0, 64)
        wl = 0.65
        src = LightSource(x, y, wl)
        src.gaussian_beam(w0=(40.0, 40.0), E0=1)
        phase = rng.uniform(-np.pi, np.pi, (64, 64))
        mod, _ = oe.SLM(src, phase, 64)
        out_p, qf_p = mod.RS_propagation(3000.0)
        out_n, qf_n = mod.RS_propagation(-2500.0)
        _save("rs_square", x=x, y=y, wavelength=wl, phase=phase, source=src.field,
              field_in=mod.field, z_pos=3000.0, out_pos=out_p.field, qf_pos=qf_p,
              z_neg=-2500.0, out_neg=out_n.field, qf_neg=qf_n)

        # 2. scalar RS of a complex random input on another grid (the reference's
        # build_grid only supports nx == ny: it reuses the x sign pattern for y).
        x = np.linspace(-150.0, 150.0, 48)
        y = np.linspace(-150.0, 150.0, 48)
        f_in = rng.standard_normal((48, 48)) + 1j * rng.standard_normal((48, 48))
        light = ScalarLight(x, y, 0.532)
        light.field = f_in
        out, qf = light.RS_propagation(1800.0)
        _save("rs_complex", x=x, y=y, wavelength=0.532, field_in=f_in, z=1800.0, out=out.field, qf=qf)

        # 3. scalar RS, odd N.
        x, y = tb.space(120.0, 63)
        f_in = rng.standard_normal((63, 63)) + 1j * rng.standard_normal((63, 63))
        light = ScalarLight(x, y, 0.633)
        light.field = f_in
        out, qf = light.RS_propagation(2200.0)
        _save("rs_odd", x=x, y=y, wavelength=0.633, field_in=f_in, z=2200.0, out=out.field, qf=qf)

        # 4. VRS behind a per-pixel LCD and a per-pixel linear polarizer.
        x, y = tb.space(160.0, 64)
        wl = 0.633
        pls = PolarizedLightSource(x, y, wl)
        pls.gaussian_beam(w0=(50.0, 50.0), jones_vector=(1, 0.5))
        eta = rng.uniform(0, 2 * np.pi, (64, 64))
        theta = rng.uniform(0, 2 * np.pi, (64, 64))
        alpha = rng.uniform(0, np.pi) * np.ones((64, 64))
        l1 = oe.LCD(pls, eta, theta)
        l2 = oe.linear_polarizer(l1, alpha)
        vout, vqf = l2.VRS_propagation(2500.0)
        _save("vrs", x=x, y=y, wavelength=wl, Ex0=pls.Ex, Ey0=pls.Ey, eta=eta, theta=theta, alpha=alpha,
              lcd_Ex=l1.Ex, lcd_Ey=l1.Ey, lcd_Ez=l1.Ez, lp_Ex=l2.Ex, lp_Ey=l2.Ey, lp_Ez=l2.Ez,
              z=2500.0, Ex=vout.Ex, Ey=vout.Ey, Ez=vout.Ez, qf=vqf)

        # 5. scalar CZT with the default output grid, and to a non-square ROI.
        x, y = tb.space(150.0, 64)
        wl = 0.532
        src = LightSource(x, y, wl)
        src.gaussian_beam(w0=(45.0, 45.0), E0=1)
        ph = rng.uniform(-np.pi, np.pi, (64, 64))
        mod, _ = oe.SLM(src, ph, 64)
        c_def = mod.CZT(4000.0)
        xo = np.linspace(-40.0, 40.0, 48)
        yo = np.linspace(-30.0, 30.0, 40)
        c_roi = mod.CZT(4000.0, xo, yo)
        _save("czt", x=x, y=y, wavelength=wl, field_in=mod.field, z=4000.0, out_default=c_def.field,
              xout=xo, yout=yo, out_roi=c_roi.field)

        # 6. vectorial CZT.
        x, y = tb.space(150.0, 64)
        Ex = rng.standard_normal((64, 64)) + 1j * rng.standard_normal((64, 64))
        Ey = rng.standard_normal((64, 64)) + 1j * rng.standard_normal((64, 64))
        vl = VectorizedLight(x, y, 0.65)
        vl.Ex, vl.Ey = Ex, Ey
        xo = np.linspace(-60.0, 60.0, 32)
        yo = np.linspace(-50.0, 50.0, 40)
        vc = vl.VCZT(3500.0, xo, yo)
        _save("vczt", x=x, y=y, wavelength=0.65, Ex_in=Ex, Ey_in=Ey, z=3500.0, xout=xo, yout=yo,
              Ex=vc.Ex, Ey=vc.Ey, Ez=vc.Ez)

        # 7. high-NA objective lens and VCZT through it.
        x, y = tb.space(1500.0, 64)
        wl = 0.65
        radius = 1800.0
        f = radius / 0.9
        pls = PolarizedLightSource(x, y, wl)
        pls.gaussian_beam(w0=(1200.0, 1200.0), jones_vector=(1, 0.3))
        a_ph = rng.uniform(0, 2 * np.pi, (64, 64))
        p_ph = rng.uniform(0, 2 * np.pi, (64, 64))
        mod = oe.sSLM(pls, a_ph, p_ph)
        lens_out, smax = oe.high_NA_objective_lens(mod, radius, f)
        xo, yo = tb.space(1.0, 32)
        foc = oe.VCZT_objective_lens(mod, radius, f, xo, yo)
        _save("high_na", x=x, y=y, wavelength=wl, radius=radius, f=f, Ex_in=mod.Ex, Ey_in=mod.Ey,
              lens_out=lens_out, sin_theta_max=smax, xout=xo, yout=yo, Ex=foc.Ex, Ey=foc.Ey, Ez=foc.Ez)

        # 8. masks and sources.
        x, y = tb.space(150.0, 48)
        wl = 0.633
        g = LightSource(x, y, wl)
        g.gaussian_beam(w0=(40.0, 55.0), E0=1.5, center=(10.0, -5.0), z_w0=(300.0, 200.0), alpha=0.3)
        pw = LightSource(x, y, wl)
        pw.plane_wave(A=2.0, theta=0.01, phi=0.7, z0=3.0)
        pg = PolarizedLightSource(x, y, wl)
        pg.gaussian_beam(w0=(40.0, 40.0), jones_vector=(1, 1j), center=(3.0, 4.0))
        al = rng.uniform(0, 2 * np.pi, (48, 48))
        phi = rng.uniform(0, 2 * np.pi, (48, 48))
        A1 = rng.uniform(0, 1, (48, 48))
        A2 = rng.uniform(0, 1, (48, 48))
        s1 = oe.sSLM(pg, al, phi)
        s2 = oe.sSLM_with_amplitude(pg, al, phi, A1, A2)
        l_sc, lmask = oe.lens(g, (120.0, 100.0), (2000.0, 2500.0))
        vl = VectorizedLight(x, y, wl)
        vl.Ex, vl.Ey, vl.Ez = pg.Ex, pg.Ey, pg.Ex * 0.1
        l_v, _ = oe.lens(vl, (120.0, 120.0), (3000.0, 3000.0))
        lcd_s = oe.LCD(vl, 1.1, 0.4)
        _save("masks", x=x, y=y, wavelength=wl, gauss=g.field, plane=pw.field, pol_Ex=pg.Ex, pol_Ey=pg.Ey,
              pol_Ez=pg.Ez, alpha=al, phi=phi, A1=A1, A2=A2, sslm_Ex=s1.Ex, sslm_Ey=s1.Ey,
              sslma_Ex=s2.Ex, sslma_Ey=s2.Ey, lens_scalar=l_sc.field, lens_mask=lmask,
              vin_Ez=vl.Ez, lens_vec_Ex=l_v.Ex, lens_vec_Ey=l_v.Ey, lens_vec_Ez=l_v.Ez,
              lcd_scalar_Ex=lcd_s.Ex, lcd_scalar_Ey=lcd_s.Ey, lcd_scalar_Ez=lcd_s.Ez)

        # 9. losses.
        a = rng.standard_normal((40, 40)) + 1j * rng.standard_normal((40, 40))
        b = rng.standard_normal((40, 40)) + 1j * rng.standard_normal((40, 40))
        I = np.abs(rng.standard_normal((40, 40))) ** 3
        _save("losses", a=a, b=b, mse_intensity=lf.MSE_Intensity(a, b), I=I,
              small_area=lf.small_area_hybrid(I))

        # 10. building block: sSLM -> VRS -> LCD.
        x, y = tb.space(150.0, 48)
        pg = PolarizedLightSource(x, y, 0.633)
        pg.gaussian_beam(w0=(40.0, 40.0), jones_vector=(1, 0))
        al = rng.uniform(0, 2 * np.pi, (48, 48))
        phi = rng.uniform(0, 2 * np.pi, (48, 48))
        bb = oe.building_block(pg, al, phi, 2000.0, np.pi / 2, np.pi / 4)
        _save("building_block", x=x, y=y, wavelength=0.633, Ex_in=pg.Ex, Ey_in=pg.Ey, alpha=al, phi=phi,
              z=2000.0, eta=np.pi / 2, theta=np.pi / 4, Ex=bb.Ex, Ey=bb.Ey, Ez=bb.Ez)

        # 11. a 4f-style table: SLM -> RS -> lens -> CZT(ROI) -> SLM -> CZT, intensity + MSE.
        x, y = tb.space(200.0, 64)
        wl = 0.532
        f4 = 6000.0
        src = LightSource(x, y, wl)
        src.gaussian_beam(w0=(80.0, 80.0), E0=1)
        p1 = rng.uniform(-np.pi, np.pi, (64, 64))
        l1, _ = oe.SLM(src, p1, 64)
        l2, _ = l1.RS_propagation(f4)
        l3, _ = oe.lens(l2, (200.0, 200.0), (f4, f4))
        xo, yo = tb.space(60.0, 32)
        l4 = l3.CZT(f4, xo, yo)
        p2 = rng.uniform(-np.pi, np.pi, (32, 32))
        l5, _ = oe.SLM(l4, p2, 32)
        l6 = l5.CZT(f4)
        I = np.abs(l6.field) ** 2
        target = (rng.uniform(0, 1, (32, 32)) < 0.1).astype(np.float64)
        _save("four_f", x=x, y=y, wavelength=wl, f=f4, source=src.field, phase1=p1, xout=xo, yout=yo,
              phase2=p2, after_rs=l2.field, after_lens=l3.field, after_czt1=l4.field, out=l6.field,
              intensity=I, target=target)

        # 12. beam splitters (lossy symmetric, single input on both ports,
        # lossless) and the fluorescence model.
        x, y = tb.space(120.0, 40)
        wl = 0.65
        la = VectorizedLight(x, y, wl)
        lb = VectorizedLight(x, y, wl)
        la.Ex = rng.standard_normal((40, 40)) + 1j * rng.standard_normal((40, 40))
        la.Ey = rng.standard_normal((40, 40)) + 1j * rng.standard_normal((40, 40))
        lb.Ex = rng.standard_normal((40, 40)) + 1j * rng.standard_normal((40, 40))
        lb.Ey = rng.standard_normal((40, 40)) + 1j * rng.standard_normal((40, 40))
        th = 0.7
        c, d = oe.BS_symmetric(la, lb, th)
        c0, d0 = oe.BS_symmetric_SI(la, th, port=0)
        c1, d1 = oe.BS_symmetric_SI(la, -2.2, port=1)
        b1, b2 = oe.BS(la, lb, 0.3, 0.7, 1.1)
        i_ex = np.abs(rng.standard_normal((3, 40, 40))) ** 2
        i_dep = np.abs(rng.standard_normal((3, 40, 40))) ** 2
        fl = oe.fluorescence(i_ex[0], i_dep[0], beta=0.8)
        vfl = oe.vectorized_fluorophores(i_ex, i_dep)
        _save("beam_splitters", x=x, y=y, wavelength=wl, aEx=la.Ex, aEy=la.Ey, bEx=lb.Ex, bEy=lb.Ey, theta=th,
              cEx=c.Ex, cEy=c.Ey, cEz=c.Ez, dEx=d.Ex, dEy=d.Ey, dEz=d.Ez,
              si0_cEx=c0.Ex, si0_cEy=c0.Ey, si0_dEx=d0.Ex, si0_dEy=d0.Ey, theta_si1=-2.2,
              si1_cEx=c1.Ex, si1_cEy=c1.Ey, si1_dEx=d1.Ex, si1_dEy=d1.Ey,
              R=0.3, T=0.7, phase=1.1, b1Ex=b1.Ex, b1Ey=b1.Ey, b2Ex=b2.Ex, b2Ey=b2.Ey,
              i_ex=i_ex, i_dep=i_dep, beta=0.8, fluorescence=fl, vfluorophores=vfl)

        # 13. the prebuilt hybrid tables on a small grid (32 x 32, 16 x 16 focus).
        n = 32
        x, y = tb.space(2500.0, n)
        xo, yo = tb.space(10.0, 16)
        r_lens, f_lens = 1800.0, 2000.0
        red = PolarizedLightSource(x, y, 0.65)
        red.gaussian_beam(w0=(1200.0, 1200.0), jones_vector=(1, 1))
        green = PolarizedLightSource(x, y, 0.532)
        green.gaussian_beam(w0=(1200.0, 1200.0), jones_vector=(1, -1))

        def scal(k):
            return rng.uniform(0, 1, (k, 1))

        p_sharp = [rng.uniform(0, 1, (n, n)) if (k % 6) in (0, 1) and k < 18 else scal(1)[0] for k in range(29)]
        i_sharp, _ = oe.hybrid_setup_sharp_focus(red, red, red, red, red, red, p_sharp, [r_lens, f_lens, xo, yo])
        i_sted = oe.hybrid_setup_fluorophores(red, green, red, green, red, green, p_sharp, [r_lens, f_lens, xo, yo],
                                              distance_offset=10)
        pms = [rng.uniform(-np.pi, np.pi, (n, n)) for _ in range(6)]
        p_fixed = [scal(1)[0] for _ in range(25)]
        fixed = [r_lens, f_lens, xo, yo] + pms
        i_fixed, _ = oe.hybrid_setup_fixed_slms(red, red, red, red, red, red, p_fixed, fixed)
        i_fixed_sted = oe.hybrid_setup_fixed_slms_fluorophores(red, green, red, green, red, green, p_fixed, fixed)
        p_robust = [rng.uniform(0, 1, (n, n)) if (k % 8) in (0, 1, 2, 3) and k < 24 else scal(1)[0]
                    for k in range(35)]
        nz = [rng.normal(0, 50.0, 1) for _ in range(8)]
        ns = [rng.normal(0, 0.1, (n, n)) for _ in range(6)]
        nw = [rng.normal(0, 0.05, 1) for _ in range(6)]
        na = [rng.normal(0, 0.02, (n, n)) for _ in range(6)]
        i_robust = oe.robust_discovery(red, red, red, red, red, red, p_robust, [r_lens, f_lens, xo, yo], nz, ns, nw, na)
        p_six = [scal(1)[0] for _ in range(52)]
        six_fixed = [r_lens, f_lens, xo, yo] + pms[:4]
        i_six = oe.six_times_six_ansatz(*([red] * 12), p_six, six_fixed, distance_offset=9.5)
        _save("hybrid_tables", x=x, y=y, xout=xo, yout=yo, r=r_lens, f=f_lens, red_Ex=red.Ex, red_Ey=red.Ey,
              green_Ex=green.Ex, green_Ey=green.Ey,
              **{f"p_sharp_{k}": v for k, v in enumerate(p_sharp)}, i_sharp=i_sharp, i_sted=i_sted,
              **{f"pm_{k}": v for k, v in enumerate(pms)}, **{f"p_fixed_{k}": v for k, v in enumerate(p_fixed)},
              i_fixed=i_fixed, i_fixed_sted=i_fixed_sted,
              **{f"p_robust_{k}": v for k, v in enumerate(p_robust)},
              **{f"noise_d_{k}": v for k, v in enumerate(nz)}, **{f"noise_s_{k}": v for k, v in enumerate(ns)},
              **{f"noise_w_{k}": v for k, v in enumerate(nw)}, **{f"noise_a_{k}": v for k, v in enumerate(na)},
              i_robust=i_robust, **{f"p_six_{k}": v for k, v in enumerate(p_six)}, i_six=i_six)

        # 14. cylindrical and axicon lenses, and the geometric masks.
        x, y = tb.space(400.0, 40)
        X, Y = np.meshgrid(x, y)
        sl = LightSource(x, y, 0.6)
        sl.gaussian_beam(w0=(150.0, 150.0), E0=1)
        vl = VectorizedLight(x, y, 0.6)
        vl.Ex = rng.standard_normal((40, 40)) + 1j * rng.standard_normal((40, 40))
        vl.Ey = rng.standard_normal((40, 40)) + 1j * rng.standard_normal((40, 40))
        vl.Ez = rng.standard_normal((40, 40)) + 1j * rng.standard_normal((40, 40))
        cyl_s, cyl_mask = oe.cylindrical_lens(sl, 5000.0, 1.5, angle=0.4)
        cyl_v, _ = oe.cylindrical_lens(vl, 5000.0, 1.5, angle=0.4)
        ax_s, ax_mask = oe.axicon_lens(sl, 0.02, 1.45)
        ax_v, _ = oe.axicon_lens(vl, 0.02, 1.45)
        tri = oe.triangular_mask(X, Y, (10.0, 60.0), 20.0, 1.2, 150.0)
        rect = oe.rectangular_mask(X, Y, (15.0, -10.0), 180.0, 90.0, 30.0)
        ann = oe.annular_aperture(100.0, 300.0, X, Y)
        fg_a = oe.forked_grating(X, Y, (5.0, 5.0), 10.0, 60.0, 2, kind='Amplitude')
        fg_p = oe.forked_grating(X, Y, (5.0, 5.0), 10.0, 60.0, 2, kind='Phase')
        _save("lenses_masks", x=x, y=y, source=sl.field, vEx=vl.Ex, vEy=vl.Ey, vEz=vl.Ez,
              cyl_scalar=cyl_s.field, cyl_mask=cyl_mask, cyl_Ex=cyl_v.Ex, cyl_Ey=cyl_v.Ey, cyl_Ez=cyl_v.Ez,
              ax_scalar=ax_s.field, ax_mask=ax_mask, ax_Ex=ax_v.Ex, ax_Ey=ax_v.Ey, ax_Ez=ax_v.Ez,
              triangle=tri, rectangle=rect, annulus=ann, forked_amplitude=fg_a, forked_phase=fg_p)

        # 15. the array-level entry points: RS / VRS jit, the transfer function,
        # CZT jit, the plain Bluestein pair, Bluestein_method and the lens helper.
        from xlumina import vectorized_optics as vo
        from xlumina import wave_optics as wo
        x, y = tb.space(140.0, 36)
        wl = 0.6
        kk = 2 * np.pi / wl
        f_in = rng.standard_normal((36, 36)) + 1j * rng.standard_normal((36, 36))
        E3 = rng.standard_normal((3, 36, 36)) + 1j * rng.standard_normal((3, 36, 36))
        nx_, ny_, dx_, dy_, Xe, Ye = wo.build_grid(x, y)
        rs_jit = wo.RS_propagation_jit(f_in, 2100.0, nx_, ny_, dx_, dy_, Xe, Ye, kk)
        vrs_jit = vo.VRS_propagation_jit(E3, 2100.0, nx_, ny_, dx_, dy_, Xe, Ye, kk)
        H = wo.transfer_function_RS(2100.0, Xe, Ye, kk)
        xo = np.linspace(-30.0, 30.0, 24)
        yo = np.linspace(-20.0, 20.0, 20)
        cnx, cny, cdx, cdy, Xo, Yo, Dm, fy1, fy2, fx1, fx2 = wo.build_CZT_grid(2500.0, wl, x, y, xo, yo)
        Xg, Yg = np.meshgrid(x, y)
        czt_jit = wo.CZT_jit(f_in, 2500.0, wl, kk, cnx, cny, cdx, cdy, Xo, Yo, Xg, Yg, Dm, fy1, fy2, fx1, fx2)
        g = (Dm, fy1, fy2, fx1, fx2)
        hg = oe.build_high_NA_VCZT_grid(2000.0, 1800.0, wl, x, xo, yo)
        plain = wo.CZT_for_high_NA_jit(f_in, *hg)
        blu = wo.Bluestein_method(f_in, -12.0, 15.0, 60.0, 20)
        th = rng.uniform(0, 0.8, (36, 36))
        phv = rng.uniform(-np.pi, np.pi, (36, 36))
        Gv = rng.uniform(0, 1, (36, 36))
        lens_h = oe._high_NA_objective_lens_(np.moveaxis(E3, 0, -1), th, phv, Gv)
        _save("array_api", x=x, y=y, wavelength=wl, field=f_in, E3=E3, rs_jit=rs_jit, vrs_jit=vrs_jit, H=H,
              xout=xo, yout=yo, czt_grid=np.array(g, dtype=np.float64), czt_jit=czt_jit,
              hna_grid=np.array(hg, dtype=np.float64), plain=plain, bluestein=blu, theta=th, phi=phv, G=Gv,
              lens_helper=lens_h)

        # 16. Jones matrices, the scalar SLM phase and the single-input splitter ports.
        al, phs, et, ths, de, a1s, a2s = 0.37, -1.1, 2.3, 0.81, 0.6, 0.7, 0.45
        ph_plane = rng.uniform(-np.pi, np.pi, (12, 12))
        aEx = rng.standard_normal((8, 8)) + 1j * rng.standard_normal((8, 8))
        aEy = rng.standard_normal((8, 8)) + 1j * rng.standard_normal((8, 8))
        zero = np.zeros((8, 8), dtype=np.complex128)
        T, R = 0.83, 0.51
        p0 = oe.bs_port0(aEx, aEy, zero, zero, zero, zero, T, R)
        p1 = oe.bs_port1(aEx, aEy, zero, zero, zero, zero, T, R)
        _save("jones", alpha=al, phi=phs, eta=et, theta=ths, delta=de, a1=a1s, a2=a2s,
              lp=oe.jones_LP(al), retarder=oe.jones_general_retarder(et, ths, de), sslm=oe.jones_sSLM(al, phs),
              sslm_amp=oe.jones_sSLM_with_amplitude(al, phs, a1s, a2s), lcd=oe.jones_LCD(et, ths),
              phase_plane=ph_plane, slm_phase=oe.phase_scalar_SLM(ph_plane), aEx=aEx, aEy=aEy, T=T, R=R,
              port0=np.stack(p0), port1=np.stack(p1))

        # 17. amplitude and phase losses, per component, and the hybrid area loss over a stack.
        import types
        a3 = rng.standard_normal((3, 20, 20)) + 1j * rng.standard_normal((3, 20, 20))
        b3 = rng.standard_normal((3, 20, 20)) + 1j * rng.standard_normal((3, 20, 20))
        la = types.SimpleNamespace(Ex=a3[0], Ey=a3[1], Ez=a3[2])
        lb = types.SimpleNamespace(Ex=b3[0], Ey=b3[1], Ez=b3[2])
        I6 = np.abs(rng.standard_normal((6, 20, 20))) ** 3
        _save("losses_more", a3=a3, b3=b3, mse_amplitude=lf.MSE_Amplitude(a3[0], b3[0]),
              mse_phase=lf.MSE_Phase(a3[0], b3[0]), vmse_amplitude=lf.vMSE_Amplitude(la, lb),
              vmse_phase=lf.vMSE_Phase(la, lb), I6=I6, loss_hybrid=lf.vectorized_loss_hybrid(I6))


    # 18. host helpers: build_CZT_grid and the minimum trustworthy RS / VRS
    # distances (get_RS_minimum_z / get_VRS_minimum_z print the value and
    # return None; the printed number is captured).
    from xlumina import wave_optics as wo

    def printed(fn):
        buf = io.StringIO()
        with contextlib.redirect_stdout(buf):
            ret = fn()
        return ret, float(buf.getvalue().split(":")[-1])

    grids = []
    for (z, wl, nin, hin, nxo, nyo, hxo, hyo) in ((2500.0, 0.6, 36, 140.0, 24, 20, 30.0, 20.0),
                                                   (5.0e4, 0.532, 64, 750.0, 32, 32, 400.0, 400.0)):
        xin, yin = tb.space(hin, nin)
        xo, yo = np.linspace(-hxo, hxo, nxo), np.linspace(-hyo, hyo, nyo)
        cnx, cny, cdx, cdy, Xo, Yo, Dm, fy1, fy2, fx1, fx2 = wo.build_CZT_grid(z, wl, xin, yin, xo, yo)
        grids.append(dict(z=z, wl=wl, xin=xin, yin=yin, xo=xo, yo=yo, scal=np.array(
            [cnx, cny, cdx, cdy, Dm, fy1, fy2, fx1, fx2], dtype=np.float64), Xo=Xo, Yo=Yo))
    minz = []
    for (h, n, wl, nidx, qf) in ((150.0, 64, 0.65, 1, 1), (1000.0, 1024, 0.633, 1, 2), (500.0, 128, 0.532, 1.5, 1),
                                 (5.0, 16, 0.6, 1, 1), (0.5, 64, 0.6, 1, 1)):
        xx, yy = tb.space(h, n)
        sl = ScalarLight(xx, yy, wl)
        ret_s, zs = printed(lambda: sl.get_RS_minimum_z(n=nidx, quality_factor=qf))
        vl = VectorizedLight(xx, yy, wl)
        ret_v, zv = printed(lambda: vl.get_VRS_minimum_z(n=nidx, quality_factor=qf))
        assert ret_s is None and ret_v is None
        minz.append((h, n, wl, nidx, qf, zs, zv))
    _save("host_helpers", **{f"g{i}_{k}": v for i, g in enumerate(grids) for k, v in g.items()},
          minz=np.array(minz, dtype=np.float64))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("XLUMINA_REF", ""))
