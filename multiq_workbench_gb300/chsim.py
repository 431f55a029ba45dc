"""The chsim command line over this engine (simulation/chsim/src/channel.rs:508-767, check.rs:62-121):
the subcommands that drive ``Engine::run_batch`` and the field diagnostics around them.

``python -m multiq_workbench_gb300.chsim <sub> [args]``:

  field                      r0_eff(z) of the RF basis and the Fig. 4 DC potential on the axis
  secular                    trajectory secular frequencies of m/z 863 and 500 (full and half force)
  legacy-fig4 [nions]        the legacy m/z scan of Fig. 4 (26 m/z x nions ions, one batch)
  s14 [Pa n barrier vac variant hole]
                             gate open / closed and the AC scan of fig. S14 (one batch)
  check-tiled [n]            every ion of a batch equals the same job run alone, bit for bit
  hash [n]                   FNV-1a hashes of the final states of fixed jobs (regression values)
  field-check                RF-only solves at 0.1 / 0.05 mm, tilted and straight, with r0_eff(z)

Global flags: ``--f64`` runs the FP64 kernel instead of the mixed engine, ``--device D`` picks the
GPU (field solves too), ``--untiled`` is accepted for compatibility (the engine has one path).
``compare-theirs`` needs the authors' exported potentials, which are not distributed.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import sys
import time

import numpy as np

from . import _native as N
from . import check
from .channel import Engine, Job, Physics, RfAc, Species, PREC_F64, PREC_MIXED
from .grid import Fields, Geom, near_window

QE, AMU = 1.602176634e-19, 1.6605390666e-27
FIG4_DC = [0.0, 5.0, -5.0, 0.0]
FIG4_DRIVE = RfAc(100.0, 500e3, 0.5, 100e3)


def fwhm(xs, ys) -> tuple:
    """Peak x, peak y and FWHM of a peaked curve by linear interpolation (channel.rs:511-520)."""
    im, ym = 0, -math.inf
    for i, y in enumerate(ys):
        if y > ym:
            ym, im = y, i
    half = ym / 2.0
    lo, hi = xs[0], xs[-1]
    for i in range(im, 0, -1):
        if ys[i - 1] < half:
            lo = xs[i - 1] + (half - ys[i - 1]) / (ys[i] - ys[i - 1]) * (xs[i] - xs[i - 1])
            break
    for i in range(im, len(xs) - 1):
        if ys[i + 1] < half:
            hi = xs[i] + (ys[i] - half) / (ys[i] - ys[i + 1]) * (xs[i + 1] - xs[i])
            break
    return xs[im], ym, hi - lo


def r0_fit(f: Fields, z_mm: float, w: int | None = None) -> float:
    """r0_eff from a least-squares fit phi = c X Y of the RF basis in the z slice (c = -2 / r0^2),
    over the nodes within w of the axis off its two planes (channel.rs:522-544)."""
    h = f.geom.h_mm
    wn = near_window(h)
    w = wn if w is None else w
    k = int(round(z_mm / h))
    near = f.rf_phi_near
    sxy = sxx = 0.0
    for dj in range(-w, w + 1):
        for di in range(-w, w + 1):
            if di == 0 or dj == 0:
                continue
            x, y = di * h, dj * h
            p = float(near[k, wn + dj, wn + di])
            sxy += p * x * y
            sxx += (x * y) * (x * y)
    return math.sqrt(-2.0 * sxx / sxy) if sxy < 0 else float("nan")


def r0_profile(f: Fields, out=sys.stdout) -> list:
    """r0_eff(z) on +-5 nodes and the AC field on the axis (channel.rs:522-544)."""
    g = f.geom
    a = f.nx // 2
    print(f"RF field check (ideal r0 = {g.r0():.4f} mm):", file=out)
    print("   z[mm]   r0_eff[mm]   E_ac_x(axis)[V/m per V]", file=out)
    rows = []
    for zmm in (3.5, 5.0, 7.0, 9.0, 11.0, 13.0, 14.5):
        k = int(round(zmm / g.h_mm))
        r0 = r0_fit(f, zmm, 5)
        eac = float(f.ac[a + f.nx * (a + f.ny * k), 0])
        rows.append((zmm, r0, eac))
        print(f"   {zmm:5.1f}   {r0:8.4f}     {eac:8.1f}", file=out)
    return rows


def secular_freq(f: Fields, sp: Species, v_rf: float, f_rf: float, z_mm: float, half_force: bool) -> float:
    """Secular frequency [Hz] from an FP64 trajectory in the RF field alone (channel.rs:555-578)."""
    qm = sp.z * QE / (sp.mass * AMU) * (0.5 if half_force else 1.0)
    rf = np.ascontiguousarray(f.rf, np.float32)
    out = C.c_double(0.0)
    N.check(N.lib().mq_secular_freq(rf.ctypes.data, f.nx, f.ny, f.nz, f.h, f.geom.axis() * 1e-3, qm, v_rf, f_rf,
                                    z_mm * 1e-3, C.byref(out)), "mq_secular_freq")
    return float(out.value)


def s14_dc(f: Fields, barrier: float | None, verbose: bool = False) -> tuple:
    """Fig. S14 DC sets (closed, open); with a barrier the gate voltage puts the on-axis saddle
    between 14 and 19 mm ``barrier`` V above the trap (channel.rs:631-644)."""
    closed = [18.0, 24.0, 15.0, 20.0]
    if barrier is not None:
        def saddle(vg):
            return max(p for z, p in f.dc_phi_axis([18.0, vg, 15.0, 20.0]) if 14.0 < z < 19.0)
        lo, hi = 20.0, 2000.0
        for _ in range(60):
            mid = 0.5 * (lo + hi)
            if saddle(mid) < 20.0 + barrier:
                lo = mid
            else:
                hi = mid
        closed[1] = hi
        if verbose:
            print(f"barrier-matched gate: {hi:.1f} V gives on-axis saddle {saddle(hi):.2f} V ({barrier} V above trap)")
    return closed, [18.0, 19.0, 15.0, 20.0]


BAK2 = Species(2.0 * 862.974, 2.0, 425.0)   # channel.rs:629


def _engine(f: Fields, f64: bool, device: int) -> Engine:
    return Engine(f, PREC_F64 if f64 else PREC_MIXED, device=device)


def cmd_field(f: Fields) -> None:
    r0_profile(f)
    print("Fig.4 DC config on axis (Q1 0, plate +5, downstream -5, box 0):")
    for z, p in f.dc_phi_axis(FIG4_DC)[::10]:
        print(f"   z {z:5.1f} mm  phi {p:7.3f} V")


def cmd_secular(f: Fields) -> None:
    bak = Species(1725.95, 2.0, 425.0)
    for zmm, label in ((5.0, "near entrance"), (9.0, "mid"), (13.0, "near exit")):
        fc = secular_freq(f, bak, 75.0, 500e3, zmm, False)
        fl = secular_freq(f, bak, 75.0, 500e3, zmm, True)
        print(f"m/z 863 @ 75 V, z = {zmm:4.1f} mm ({label}): f_sec correct {fc / 1e3:6.2f} kHz | legacy half-force "
              f"{fl / 1e3:6.2f} kHz | S14 used 83 kHz")
    m500 = Species(500.0, 1.0, 230.0)
    fc = secular_freq(f, m500, 100.0, 500e3, 9.0, False)
    fl = secular_freq(f, m500, 100.0, 500e3, 9.0, True)
    print(f"m/z 500 @ 100 V (Fig. 4 point), mid: correct {fc / 1e3:.2f} kHz (expected unstable) | legacy "
          f"{fl / 1e3:.2f} kHz (their 100 kHz)")


def fig4_jobs(nions: int, first: float = 475.0, last: float = 525.0) -> list:
    mzs = [first + 2.0 * i for i in range(int((last - first) / 2.0) + 1)]
    return [Job(Species(mz * 5.0, 5.0, 0.0), FIG4_DRIVE, nions, 1000 + int(mz)) for mz in mzs]


def cmd_legacy_fig4(eng: Engine, nions: int) -> tuple:
    """The legacy m/z scan of Fig. 4 in one batch (channel.rs:735-759); returns (peak m/z, peak, FWHM)."""
    ph = Physics.legacy(1e-3 * 133.322)
    jobs = fig4_jobs(nions)
    print(f"Legacy replication of Fig. 4 (m/z scan, {nions} ions/point, 5+ ions of m/z = mass/5):")
    print("  m/z    returned  transmitted  collided  left  timeout   <coll>   <t>[ms]")
    t0 = time.time()
    outs = eng.run_batch(jobs, FIG4_DC, ph)
    dt = time.time() - t0
    xs, ys = [], []
    for j, o in zip(jobs, outs):
        mz = j.sp.mass / 5.0
        xs.append(mz)
        ys.append(o.transmitted / o.n)
        print(f"  {mz:5.0f}  {o.returned / o.n:7.3f}   {o.transmitted / o.n:7.3f}     {o.crashed / o.n:7.3f}  "
              f"{o.left / o.n:5.3f}  {o.timeout / o.n:5.3f}   {o.mean_coll:7.1f}  {o.mean_time * 1e3:7.3f}")
    pk, py, w = fwhm(xs, ys)
    print(f"peak {py * 100:.1f}% at m/z {pk:.0f}; FWHM {w:.1f} m/z => R = {pk / w:.0f}   (their Fig. 4: ~80%, R ~ 50)")
    print(f"scan time {dt:.3f} s (one batch of {len(jobs)} jobs)")
    return pk, py, w


def cmd_s14(args: list, f64: bool, device: int) -> tuple:
    """Fig. S14: gate open and closed without AC, and the closed-gate AC scan 70..110 kHz in one
    batch (channel.rs:646-689)."""
    def arg(i, default, conv=float):
        try:
            return conv(args[i])
        except (IndexError, ValueError):
            return default
    variant = args[5] if len(args) > 5 else "code"
    hole = arg(6, None)
    geom = Geom.s14(variant, hole_d=hole)
    print(f"geometry variant: {variant} (tilt_mode {geom.tilt_mode}, ac_mode {geom.ac_mode}, alpha {geom.alpha:.4f} "
          f"per rod, gate hole {geom.hole_d:.2f} mm)")
    f = Fields.build(geom, device=device)
    pa, n = arg(1, 0.1), arg(2, 2000, int)
    barrier = arg(3, None)
    if barrier is not None and not barrier > -50.0:
        barrier = None
    vac = arg(4, 3.0)
    ph = Physics.correct(pa)
    ph.t_max = 5e-3
    closed, opened = s14_dc(f, barrier, verbose=True)
    ax = f.dc_phi_axis(closed)
    zmax, vmax = max(((z, p) for z, p in ax if 12.0 < z < 19.0), key=lambda t: t[1])
    vmin = min(p for z, p in ax if 4.0 < z < 15.0)
    print(f"S14 config on axis: trap side 20 V, channel well min {vmin:.2f} V, gate max {vmax:.2f} V at "
          f"z={zmax:.1f} mm (=> {vmax - 20.0:.2f} V above trap)")

    def rf(v_ac, f_ac=83e3):
        return RfAc(75.0, 500e3, v_ac, f_ac)
    with _engine(f, f64, device) as eng:
        o_open = eng.run_batch([Job(BAK2, rf(0.0), n, 7)], opened, ph)[0]
        fs = [70.0 + i for i in range(41)]
        jobs = [Job(BAK2, rf(0.0), 1 if os.environ.get("CHSIM_S14_NONOAC") else n, 8)]
        jobs += [Job(BAK2, rf(vac, fk * 1e3), n, 100 + int(fk)) for fk in fs]
        t0 = time.time()
        outs_all = eng.run_batch(jobs, closed, ph)
        dt = time.time() - t0
    o_noac, outs = outs_all[0], list(outs_all)[1:]

    def fr(o, k):
        return getattr(o, k) / max(o.n, 1)
    print(f"Bak BH3 2+ (m/z 863.0), {pa} Pa, {n} ions/pt, per pass from trap side:")
    print(f"  gate OPEN, no AC:    transmitted {fr(o_open, 'transmitted'):.3f}  returned {fr(o_open, 'returned'):.3f}  "
          f"crashed {fr(o_open, 'crashed'):.3f}  in-channel@{ph.t_max * 1e3:g}ms {fr(o_open, 'timeout'):.3f}")
    print(f"  gate CLOSED, no AC:  transmitted {fr(o_noac, 'transmitted'):.3f}  returned {fr(o_noac, 'returned'):.3f}  "
          f"crashed {fr(o_noac, 'crashed'):.3f}  in-channel {fr(o_noac, 'timeout'):.3f}")
    print(f"  gate CLOSED, AC {vac} V (per side) scan:")
    print("   f[kHz]  transm  return  crash  in-ch  <coll>  <t>[ms]   eff_ss=T/(T+C)")
    xs, ys = [], []
    for fk, o in zip(fs, outs):
        tr, cr = fr(o, "transmitted"), fr(o, "crashed")
        eff = tr / (tr + cr) if tr + cr > 0 else 0.0
        print(f"   {fk:5.1f}   {tr:.3f}   {fr(o, 'returned'):.3f}   {cr:.3f}  {fr(o, 'timeout'):.3f}  {o.mean_coll:6.1f}  "
              f"{o.mean_time * 1e3:6.3f}    {eff:.3f}")
        xs.append(fk)
        ys.append(tr)
    pk, py, w = fwhm(xs, ys)
    print(f"resonance: peak {py * 100:.1f}% per pass at {pk:.1f} kHz (their S14 setting: 83 kHz); FWHM {w:.1f} kHz "
          f"=> f/df = {pk / w:.1f}")
    print(f"scan time {dt:.3f} s ({len(jobs)} jobs x {n} ions = {len(jobs) * n} ions in one batch)")
    return pk, py, w


def cmd_check_tiled(n: int, f64: bool, device: int) -> int:
    """Every ion of each batch equals the same job run alone (check.rs:62-92 job sets); returns the
    number of differing ions."""
    bad = 0
    f = Fields.build(Geom(), device=device)
    with _engine(f, f64, device) as eng:
        ph = Physics.legacy(1e-3 * 133.322)
        jobs = [Job(Species(mz * 5.0, 5.0, 0.0), FIG4_DRIVE, n, 1000 + int(mz)) for mz in (475.0 + 2.0 * i for i in range(26))]
        ph2 = Physics.legacy(1e-3 * 133.322)
        ph2.legacy_fields = False
        ph3 = Physics.correct(0.1)
        ph3.legacy_fields = True
        ph3.t_max = 2e-3
        jobs3 = [Job(BAK2, RfAc(75.0, 500e3, 1.0, (70.0 + 4.0 * i) * 1e3), n, 50 + i) for i in range(6)]
        for label, js, dc, p in (("legacy Fig.4", jobs, FIG4_DC, ph),
                                 ("legacy collisions + trilinear fields", jobs[8:14], FIG4_DC, ph2),
                                 ("thermal gas + nearest-node fields", jobs3, [18.0, 24.0, 15.0, 20.0], ph3)):
            d = check.check_case(eng, js, dc, p)
            print(f"[{label}] {len(js)} jobs, {d['n']} ions: {d['differ']} / {d['n']} ions differ from the jobs run alone")
            bad += d["differ"]
    fs14 = Fields.build(Geom.s14(), device=device)
    with _engine(fs14, f64, device) as eng:
        ph = Physics.correct(0.1)
        ph.t_max = 5e-3
        closed, opened = s14_dc(fs14, None)
        jobs = [Job(BAK2, RfAc(75.0, 500e3, 1.5, fk * 1e3), n, 100 + fk) for fk in range(70, 97)]
        for label, js, dc in (("S14 closed gate, AC 1.5 V scan", jobs, closed),
                              ("S14 gate open, no AC", [Job(BAK2, RfAc(75.0, 500e3, 0.0, 83e3), n * 4, 7)], opened)):
            d = check.check_case(eng, js, dc, ph)
            print(f"[{label}] {len(js)} jobs, {d['n']} ions: {d['differ']} / {d['n']} ions differ from the jobs run alone")
            bad += d["differ"]
    print("check-tiled: PASS (bitwise identical final states)" if bad == 0 else "check-tiled: FAIL")
    return bad


def cmd_hash(n: int, f64: bool, device: int) -> list:
    """FNV-1a hashes of the final states of fixed single jobs (check.rs:97-121).  The state layout
    is this engine's, so the values are regression values of this engine, not chsim's."""
    out = []
    f = Fields.build(Geom(), device=device)
    with _engine(f, f64, device) as eng:
        ph = Physics.legacy(1e-3 * 133.322)
        for mz in (475.0, 491.0, 499.0, 507.0, 523.0):
            print(f"legacy mz {mz:g}")
            ions, _ = eng.run_batch_ions([Job(Species(mz * 5.0, 5.0, 0.0), FIG4_DRIVE, n, 1000 + int(mz))], FIG4_DC, ph)
            h = check.hash_ions(ions)
            out.append(h)
            print(f"HASH {h:016x} n={n}")
    fs14 = Fields.build(Geom.s14(), device=device)
    with _engine(fs14, f64, device) as eng:
        ph = Physics.correct(0.1)
        ph.t_max = 5e-3
        closed, _ = s14_dc(fs14, None)
        for fk in (75.0, 81.0, 83.0, 90.0):
            print(f"s14 f {fk:g}")
            ions, _ = eng.run_batch_ions([Job(BAK2, RfAc(75.0, 500e3, 1.5, fk * 1e3), n, 100 + int(fk))], closed, ph)
            h = check.hash_ions(ions)
            out.append(h)
            print(f"HASH {h:016x} n={n}")
    return out


def cmd_field_check(device) -> None:
    """RF(+AC) solves at 0.1 / 0.05 mm, tilted (0.02 rad per rod) and straight, r0_eff(z) from a fit
    within 0.5 mm of the axis (channel.rs:580-602)."""
    for h, al in ((0.1, 0.02), (0.05, 0.02), (0.1, 0.0), (0.05, 0.0)):
        g = Geom(h_mm=h, n_xy=int(round(16.0 / h)), alpha=al)
        t0 = time.time()
        f = Fields.build(g, bases=[0, 1], cache=False, device=device)
        vals = "  ".join(f"z{z:.1f}:{r0_fit(f, z):.4f}" for z in (3.5, 5.0, 7.0, 9.0, 11.0, 13.0, 14.5))
        print(f"h={h:.3f} mm alpha={al:.3f}: r0_eff(z) =  {vals}   ({time.time() - t0:.1f} s, {f.nx}x{f.ny}x{f.nz})")


USAGE = ("channel subcommands: field | secular | legacy-fig4 [nions] | s14 [Pa n barrier vac variant hole] | "
         "check-tiled [n] | hash [n] | field-check   (flags: --f64, --device D, --untiled)")


def main(argv=None) -> int:
    args = list(sys.argv[1:] if argv is None else argv)
    f64 = "--f64" in args
    device = 0
    if "--device" in args:
        i = args.index("--device")
        device = int(args[i + 1])
        del args[i:i + 2]
    args = [a for a in args if a not in ("--f64", "--untiled")]
    sub = args[0] if args else ""

    def num(i, default, conv=int):
        try:
            return conv(args[i])
        except (IndexError, ValueError):
            return default
    if sub == "compare-theirs":
        print("compare-theirs needs the authors' exported potentials (eject_*.f32), which are not distributed")
        return 1
    if sub == "s14":
        cmd_s14(args, f64, device)
        return 0
    if sub == "check-tiled":
        return 1 if cmd_check_tiled(num(1, 300), f64, device) else 0
    if sub == "hash":
        cmd_hash(num(1, 300), f64, device)
        return 0
    if sub == "field-check":
        cmd_field_check(device)
        return 0
    if sub in ("field", "secular", "legacy-fig4"):
        f = Fields.build(Geom(), device=device if sub == "legacy-fig4" else None)
        if sub == "field":
            cmd_field(f)
        elif sub == "secular":
            cmd_secular(f)
        else:
            with _engine(f, f64, device) as eng:
                cmd_legacy_fig4(eng, num(1, 1000))
        return 0
    print(USAGE, file=sys.stderr)
    return 2


if __name__ == "__main__":
    raise SystemExit(main())
