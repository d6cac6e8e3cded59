"""The sweep workloads this engine is measured and checked on.

Each builder takes an `api` namespace with mom25d's layout classes
(`Layout`, `Substrate`, `Stackup`, `Dielectric`, `CoplanarGround`) so the
same geometry can be built with this package or with mom25d itself, and
returns (layout, stack, mesh keyword arguments, frequencies [Hz]).

  tee        open-stub tee, eps_r 3.55 / 0.508 mm, mesh 0.5/0.08 mm, 37 f 1-10 GHz (N = 1085)
  lpf        7-section stepped-impedance low-pass 4.0/0.3 mm (seeded lengths), 101 f 0.5-8 GHz;
             mesh 0.35/0.05 mm gives N = 5943, the N ~ 6k headline case
  bandpass   16 seeded edge-coupled-line band-pass variants, 128 f 1-12 GHz, each meshed with its own
             max_cell (BANDPASS_CELL) so that N spreads over 1.5k-5k (BANDPASS_N)
  via        two-layer microstrip -> via -> inner line, 2 x 0.254 mm eps_r 3.66 (N = 3789)
  gcpw       30 mm grounded CPW with via fences on 0.508 mm eps_r 3.55, 64 f 1-20 GHz
  line       short through line (small N, test case)
  line_lossless  the same line on a lossless substrate (the lossless wave fit)
  shunt_via  short line with a via to ground (small N, test case)
  lumped_line  two line sections joined by a lumped component (R 20 + L 0.5n) across a gap
  component_line  three line sections, a 2-port S-parameter block across two open gaps
  gap_port_line   a series gap in a line with an internal gap port across it
  via_port_line   a line with a via to ground fed by an internal via port
  stripline  a centred 0.4 mm stripline under a PEC cover, 2 x 0.254 mm eps_r 3.66 (mom25d's
             Engine/tests/test_multilayer.py:59-76 geometry), 2 and 10 GHz
"""

import numpy as np

mm = 1e-3
GHz = 1e9
ER, H, TAND, SIGMA = 3.55, 0.508 * mm, 0.0027, 5.8e7


def tee(api):
    W = 1.137 * mm
    lay = api.Layout()
    lay.add_rect(-W / 2 - 2 * mm, -W / 2, W / 2 + 2 * mm, W / 2)
    lay.add_rect(-W / 2, W / 2, W / 2, W / 2 + 6.6 * mm)
    lay.add_port("P1", ref=(-W / 2 - 2 * mm, 0), direction="-x", width=W, length=15 * mm)
    lay.add_port("P2", ref=(W / 2 + 2 * mm, 0), direction="+x", width=W, length=15 * mm)
    sub = api.Substrate(eps_r=ER, h=H, tand=TAND, sigma=SIGMA)
    return lay, sub, dict(max_cell=0.5 * mm, edge_cell=0.08 * mm), np.linspace(1, 10, 37) * GHz


def lpf(api, max_cell=0.35 * mm, edge_cell=0.05 * mm, seed=0):
    widths = [4.0 * mm if k % 2 == 0 else 0.3 * mm for k in range(7)]
    lengths = np.random.default_rng(seed).uniform(2.5, 5.0, 7) * mm
    lay = api.Layout()
    x = 0.0
    for w, l in zip(widths, lengths):
        lay.add_rect(x, -w / 2, x + l, w / 2)
        x += l
    W0 = 1.1366 * mm
    lay.add_port("P1", (0.0, 0.0), "-x", W0, 15 * mm)
    lay.add_port("P2", (x, 0.0), "+x", W0, 15 * mm)
    sub = api.Substrate(eps_r=ER, h=H, tand=TAND, sigma=SIGMA)
    return lay, sub, dict(max_cell=max_cell, edge_cell=edge_cell), np.linspace(0.5, 8, 101) * GHz


# max_cell [mm] of band-pass variant k, picked (0.01 mm steps) so that N comes
# near 1500 + 3500 k / 15: uneven sizes between 1.5k and 5k unknowns
BANDPASS_CELL = (0.45, 0.47, 0.44, 0.38, 0.46, 0.40, 0.38, 0.38, 0.32, 0.26, 0.28, 0.28, 0.26, 0.25, 0.22, 0.24)
BANDPASS_N = (1524, 1800, 1784, 2164, 2434, 2467, 2882, 3064, 3572, 3614, 3722, 3982, 4252, 4452, 4972, 4652)


def bandpass(api, k=0, max_cell=None, edge_cell=0.05 * mm):
    """Edge-coupled half-wave band-pass variant k: gap U(0.1, 0.4) mm,
    width U(0.8, 1.4) mm, 3-5 coupled sections, each a pair of
    quarter-wave-long rectangles offset along x; meshed with
    BANDPASS_CELL[k] unless max_cell is given."""
    rng = np.random.default_rng(k)
    gap = rng.uniform(0.1, 0.4) * mm
    W = rng.uniform(0.8, 1.4) * mm
    nsec = int(rng.integers(3, 6))
    L = 4.2 * mm  # ~quarter wave at 10 GHz on eps_eff ~2.7
    lay = api.Layout()
    x, y = 0.0, 0.0
    W0 = 1.1366 * mm
    for s in range(nsec + 1):
        lay.add_rect(x, y - W / 2, x + 2 * L, y + W / 2)
        x += L
        y += W + gap
    lay.add_port("P1", (0.0, 0.0), "-x", W, 8 * mm)
    lay.add_port("P2", (x + L, y - W - gap), "+x", W, 8 * mm)
    sub = api.Substrate(eps_r=ER, h=H, tand=TAND, sigma=SIGMA)
    mc = max_cell if max_cell is not None else BANDPASS_CELL[k] * mm
    return lay, sub, dict(max_cell=mc, edge_cell=edge_cell), np.linspace(1, 12, 128) * GHz


def via(api):
    ER2, H1, H2 = 3.66, 0.254 * mm, 0.254 * mm
    WT, WI = 1.1122 * mm, 0.45 * mm
    REF, FEED = 3 * mm, 12 * mm
    lay = api.Layout()
    lay.add_rect(-REF, -WT / 2, 0, WT / 2, layer="top")
    lay.add_rect(0, -WI / 2, REF, WI / 2, layer="inner")
    lay.add_port("P1", (-REF, 0), "-x", WT, FEED, layer="top")
    lay.add_port("P2", (REF, 0), "+x", WI, FEED, layer="inner")
    lay.add_via(0, 0, drill=0.3 * mm, pad=0.6 * mm, top="top", bottom="inner")
    st = api.Stackup([api.Dielectric(H1, ER2, 0.0037), api.Dielectric(H2, ER2, 0.0037)],
                     {"inner": 1, "top": 2}, sigma=SIGMA)
    return lay, st, dict(max_cell=0.2 * mm, edge_cell=0.05 * mm), np.linspace(1, 20, 20) * GHz


def gcpw(api, max_cell=0.15 * mm, edge_cell=0.04 * mm):
    W, G, WG = 1.137 * mm, 0.2 * mm, 1.2 * mm
    lay = api.Layout()
    lay.add_rect(-15 * mm, -W / 2, 15 * mm, W / 2)
    for sg in (1, -1):
        y0 = sg * (W / 2 + G)
        lay.add_rect(-15 * mm, y0, 15 * mm, y0 + sg * WG)
        for x in np.arange(-14.5, 15.0, 1.0) * mm:
            lay.add_via(x, y0 + sg * WG / 2, drill=0.3 * mm, pad=0.5 * mm)
    cg = api.CoplanarGround(G, WG, via_pitch=1 * mm, via_drill=0.3 * mm, via_pad=0.5 * mm)
    lay.add_port("P1", (-15 * mm, 0), "-x", W, 6 * mm, ground=cg)
    lay.add_port("P2", (15 * mm, 0), "+x", W, 6 * mm, ground=cg)
    sub = api.Substrate(eps_r=ER, h=H, tand=TAND, sigma=SIGMA)
    return lay, sub, dict(max_cell=max_cell, edge_cell=edge_cell), np.linspace(1, 20, 64) * GHz


def line(api, length=4 * mm, cell=0.5 * mm):
    W = 1.137 * mm
    lay = api.Layout()
    lay.add_rect(0, -W / 2, length, W / 2)
    lay.add_port("P1", (0, 0), "-x", W, 8 * mm)
    lay.add_port("P2", (length, 0), "+x", W, 8 * mm)
    sub = api.Substrate(eps_r=ER, h=H, tand=TAND, sigma=SIGMA)
    return lay, sub, dict(max_cell=cell, edge_cell=0.15 * mm), np.array([2.0, 7.0]) * GHz


def line_lossless(api):
    """The through line on a lossless substrate (tan d = 0, ideal
    conductors): the wave fit takes mom25d's lossless branch (gamma = j beta
    by a bounded scalar search)."""
    lay, _, mkw, freqs = line(api)
    return lay, api.Substrate(eps_r=ER, h=H), mkw, freqs


def shunt_via(api):
    W = 0.5561 * mm
    lay = api.Layout()
    lay.add_rect(-2 * mm, -W / 2, 2 * mm, W / 2)
    lay.add_port("P1", (-2 * mm, 0), "-x", W, 4 * mm)
    lay.add_port("P2", (2 * mm, 0), "+x", W, 4 * mm)
    lay.add_via(0, 0, drill=0.3 * mm, pad=W)
    sub = api.Substrate(3.66, 0.254 * mm, 0.003, SIGMA)
    return lay, sub, dict(max_cell=0.35 * mm, edge_cell=0.08 * mm), np.array([3.0, 9.0]) * GHz


def lumped_line(api, value="R 20 + L 0.5n"):
    """Two line sections joined by a lumped component across a 1 mm bridge
    (Layout.add_lumped) with a delta gap in its middle."""
    W = 1.137 * mm
    lay = api.Layout()
    lay.add_rect(0, -W / 2, 3 * mm, W / 2)
    lay.add_rect(4 * mm, -W / 2, 7 * mm, W / 2)
    lay.add_lumped("Z1", (3 * mm, 0.0), (4 * mm, 0.0), 0.6 * mm, value=value)
    lay.add_port("P1", (0, 0), "-x", W, 8 * mm)
    lay.add_port("P2", (7 * mm, 0), "+x", W, 8 * mm)
    sub = api.Substrate(eps_r=ER, h=H, tand=TAND, sigma=SIGMA)
    return lay, sub, dict(max_cell=0.5 * mm, edge_cell=0.15 * mm), np.array([2.0, 5.0, 9.0]) * GHz


def component_line(api, block=None):
    """Three line sections joined by two open lumped gaps with a 2-port
    S-parameter block (Layout.add_component, a Touchstone file) across them."""
    W = 1.137 * mm
    lay = api.Layout()
    lay.add_rect(0, -W / 2, 3 * mm, W / 2)
    lay.add_rect(4 * mm, -W / 2, 6 * mm, W / 2)
    lay.add_rect(7 * mm, -W / 2, 10 * mm, W / 2)
    lay.add_lumped("G1", (3 * mm, 0.0), (4 * mm, 0.0), 0.6 * mm)
    lay.add_lumped("G2", (6 * mm, 0.0), (7 * mm, 0.0), 0.6 * mm)
    if block is not None:
        lay.add_component(block, ["G1", "G2"])
    lay.add_port("P1", (0, 0), "-x", W, 8 * mm)
    lay.add_port("P2", (10 * mm, 0), "+x", W, 8 * mm)
    sub = api.Substrate(eps_r=ER, h=H, tand=TAND, sigma=SIGMA)
    return lay, sub, dict(max_cell=0.5 * mm, edge_cell=0.15 * mm), np.array([2.0, 5.0, 9.0]) * GHz


BUILDERS = dict(tee=tee, lpf=lpf, bandpass=bandpass, via=via, gcpw=gcpw, line=line, line_lossless=line_lossless,
                shunt_via=shunt_via,
                lumped_line=lumped_line, component_line=component_line)


def build(api, name, **kw):
    lay, stack, mkw, freqs = BUILDERS[name](api, **kw)
    return lay, stack, lay.mesh(**mkw), freqs


def gap_port_line(api):
    """A 0.5 mm series gap in a 50 ohm line on 0.254 mm eps_r 3.66 with an
    internal gap port across it (Layout.add_gap_port, z_ref 50 ohm)."""
    W, G = 0.5561 * mm, 0.5 * mm
    lay = api.Layout()
    lay.add_rect(-5 * mm, -W / 2, -G / 2, W / 2)
    lay.add_rect(G / 2, -W / 2, 5 * mm, W / 2)
    lay.add_port("P1", (-5 * mm, 0), "-x", W, 10 * mm)
    lay.add_port("P2", (5 * mm, 0), "+x", W, 10 * mm)
    lay.add_gap_port("G", (-G / 2, 0), (G / 2, 0), W)
    sub = api.Substrate(3.66, 0.254 * mm, 0.003, SIGMA)
    return lay, sub, dict(max_cell=0.4 * mm, edge_cell=0.05 * mm), np.array([1.0, 4.0, 8.0]) * GHz


def via_port_line(api):
    """A 50 ohm line with a via to ground at its middle, fed at the ground
    plane by an internal via port (Layout.add_via_port, z_ref 50 ohm)."""
    W = 0.5561 * mm
    lay = api.Layout()
    lay.add_rect(-3 * mm, -W / 2, 3 * mm, W / 2)
    lay.add_port("P1", (-3 * mm, 0), "-x", W, 6 * mm)
    lay.add_port("P2", (3 * mm, 0), "+x", W, 6 * mm)
    lay.add_via(0, 0, drill=0.3 * mm, pad=W)
    lay.add_via_port("V", 0)
    sub = api.Substrate(3.66, 0.254 * mm, 0.003, SIGMA)
    return lay, sub, dict(max_cell=0.4 * mm, edge_cell=0.05 * mm), np.array([3.0, 6.0, 9.0]) * GHz


BUILDERS.update(gap_port_line=gap_port_line, via_port_line=via_port_line)


def stripline(api):
    """A 4 mm centred stripline under a PEC cover: the 0.4 mm strip on the
    interface of two 0.254 mm eps_r 3.66 layers (mom25d's stripline check,
    Engine/tests/test_multilayer.py:59-76: eps_eff = eps_r, Z0 of the
    zero-thickness strip from K(k) / K(k'))."""
    er, hh, W = 3.66, 0.254 * mm, 0.4 * mm
    lay = api.Layout()
    lay.add_rect(-2 * mm, -W / 2, 2 * mm, W / 2, layer="mid")
    lay.add_port("P1", (-2 * mm, 0), "-x", W, 6 * mm, layer="mid")
    lay.add_port("P2", (2 * mm, 0), "+x", W, 6 * mm, layer="mid")
    st = api.Stackup([api.Dielectric(hh, er), api.Dielectric(hh, er)], {"mid": 1}, top="pec")
    return lay, st, dict(max_cell=0.25 * mm, edge_cell=0.04 * mm), np.array([2.0, 10.0]) * GHz


BUILDERS.update(stripline=stripline)
