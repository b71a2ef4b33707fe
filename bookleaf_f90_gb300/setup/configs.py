"""The workloads, written as control files in the reference's namelist format.

Each function returns the text of a deck that ``Problem.from_deck`` reads
with the reference's own rules; the decks follow the reference's input/
decks (sod_sm_lag_small, sedov_lag_small, noh_small) rescaled to the stated
domains and mesh sizes:

  sod(nx, ny)            Sod shock tube on [0,1]x[0,0.1], gamma 1.4, t=0.2
  sod_reference(nx, ny)  the same problem in the reference check's geometry
                         [0,100]x[0,10], t=20 (check_kn_tests.f90 applies)
  sedov(n)               Sedov blast, quarter domain [0,1.2]^2, gamma 1.4,
                         E=0.244816 in the corner cell, cold background 1e-12
  noh(n, eulerian)       Noh implosion on [0,1]^2, gamma 5/3, u=-r/|r|
"""


def _mesh(nx, ny, x0, y0, x1, y1, bcs):
    b, r, t, l = bcs
    return f"""&MESH
 region_typ(1)='LIN1'
 region_dim(1,:)={nx},{ny}
 region_side(1,1,:)=1,1
 region_side(1,2,:)=1,2
 region_side(1,3,:)=1,3
 region_side(1,4,:)=1,4
 segment_typ(:)='LINE','LINE','LINE','LINE'
 segment_bc(:)='{b}','{r}','{t}','{l}'
 segment_pos(1,:)={x0},{y0},{x1},{y0}
 segment_pos(2,:)={x1},{y0},{x1},{y1}
 segment_pos(3,:)={x1},{y1},{x0},{y1}
 segment_pos(4,:)={x0},{y1},{x0},{y0}
/
"""


def sod(nx=400, ny=40, time_end=0.2, eulerian=False, scale=1.0, gamma=1.4, pratio=10.0):
    """Sod shock tube.  ``gamma`` and the pressure ratio ``pratio`` of the
    left (rho 1, p 1) and right (rho 0.125, p 1/pratio) states default to the
    classic problem (e = 2.5 and 2.0)."""
    L = 1.0 * scale
    H = 0.1 * scale
    ale = "&ALE\n zeul=.TRUE.\n/\n" if eulerian else ""
    s = scale
    if gamma == 1.4 and pratio == 10.0:
        e_left, e_right = 2.5, 2.0
    else:
        e_left = 1.0 / ((gamma - 1.0) * 1.0)
        e_right = (1.0 / pratio) / ((gamma - 1.0) * 0.125)
    return f"""&CONTROL
 time_start=0.0
 time_end={time_end!r}
 dt_initial={1.0e-5 * s!r}
 dt_max={1.0e-3 * s!r}
 dt_min={1.0e-10 * s!r}
 dt_g=1.02
 cfl_sf=0.5
 cvisc1=0.5
 cvisc2=0.75
/
&EOS
 eos_type(1)='ideal gas'
 eos_param(1,1)={gamma!r}
/
""" + _mesh(nx, ny, 0.0, 0.0, L, H, ("SLIPY", "SLIPX", "SLIPY", "SLIPX")) + ale + f"""&INDICATORS
 region_type(1)='background'
 region_name(1)='air'
 region_type(2)='shape'
 region_name(2)='helium'
 region_value(2)=1
 material_type(1)='background'
 material_name(1)='shocktube'
/
&INITIAL_CONDITIONS
 thermodynamic_type(1)='region'
 thermodynamic_value(1)=1
 density(1)=1.0
 energy(1)={e_left!r}
 thermodynamic_type(2)='region'
 thermodynamic_value(2)=2
 density(2)=0.125
 energy(2)={e_right!r}
/
&SHAPES
 shape_type(1)='rectangle'
 shape_param(1,:)={0.5 * L!r},{-0.1 * L!r},{1.5 * L!r},{0.5 * L!r}
/
"""


def sod_reference(nx=100, ny=10, time_end=20.0, eulerian=False):
    """Sod in the geometry the reference's known-answer check assumes."""
    return sod(nx, ny, time_end=time_end, eulerian=eulerian, scale=100.0)


def sedov(n=512, time_end=1.0, eulerian=False, gamma=1.4, energy=0.244816, kappa=None,
          pmerit=None):
    """Sedov blast on the quarter domain [0,1.2]^2.  ``kappa`` adds the
    hourglass filter (kappaall) that the reference's own Sedov decks set
    (input/sedov_lag_small: 0.01), ``pmerit`` the sub-zonal pressure force
    (pmeritall).  Without them the Lagrangian mesh tangles at the origin
    long before t = 1 and the run stops on dt < dt_min; at 512x512 the
    hourglass filter alone is not enough (stops at t = 0.18), with
    pmeritall=0.1 as well the run reaches t = 1 in 2,800 steps."""
    ale = "&ALE\n zeul=.TRUE.\n/\n" if eulerian else ""
    hg = "" if kappa is None else f" kappaall={kappa!r}\n"
    if pmerit is not None:
        hg += f" pmeritall={pmerit!r}\n"
    return f"""&CONTROL
 time_start=0.0
 time_end={time_end!r}
 dt_initial=1.0e-4
 dt_max=1.0e-1
 dt_min=1.0e-8
 dt_g=1.02
 cfl_sf=0.5
 cvisc1=0.5
 cvisc2=0.75
{hg}/
&EOS
 eos_type(1)='ideal gas'
 eos_param(1,1)={gamma!r}
/
""" + _mesh(n, n, 0.0, 0.0, 1.2, 1.2, ("SLIPY", "FREE", "FREE", "SLIPX")) + ale + f"""&INDICATORS
 region_type(1)='background'
 region_name(1)='air'
 region_type(2)='cell'
 region_name(2)='source'
 region_value(2)=1
 material_type(1)='background'
 material_name(1)='air'
/
&INITIAL_CONDITIONS
 thermodynamic_type(1)='region'
 thermodynamic_value(1)=1
 density(1)=1.0
 energy(1)=1.0e-12
 thermodynamic_type(2)='region'
 thermodynamic_value(2)=2
 thermodynamic_energy_scale(2)='volume'
 density(2)=1.0
 energy(2)={energy!r}
/
"""


def noh(n=2048, time_end=0.6, eulerian=False):
    ale = "&ALE\n zeul=.TRUE.\n/\n" if eulerian else ""
    return f"""&CONTROL
 time_start=0.0
 time_end={time_end!r}
 dt_initial=1.0e-4
 dt_max=1.0e-2
 dt_min=1.0e-8
 dt_g=1.02
 cfl_sf=0.5
 cvisc1=0.5
 cvisc2=0.75
/
&EOS
 eos_type(1)='ideal gas'
 eos_param(1,1)=1.6666667
/
&CUTOFF
 zcut=1.0e-40
 accut=1.0e-40
 pcut=1.0e-40
/
""" + _mesh(n, n, 0.0, 0.0, 1.0, 1.0, ("SLIPY", "FREE", "FREE", "SLIPX")) + ale + """&INDICATORS
 region_type(1)='background'
 region_name(1)='air'
 material_type(1)='background'
 material_name(1)='air'
/
&INITIAL_CONDITIONS
 thermodynamic_type(1)='region'
 thermodynamic_value(1)=1
 density(1)=1.0
 energy(1)=0.0
 kinematic_type(1)='background'
 kinematic_value(1)=1
 kinematic_geometry(1)='radial'
 kinematic_param(1,1)=-1.0
 kinematic_param(2:3,1)=0.0
/
"""


def noh_polar(nr=1800, ntheta=720, time_end=0.6):
    """Noh on the reference's own polar mesh (input/noh_small, noh_large):
    one LIN2 region over the quarter annulus 0.005 <= r <= 1 with nr cells
    along the radius and ntheta around, straight sides on the axes (SLIPY,
    SLIPX), an ARC_A outer side (FREE) and an ARC_C inner side (WALL);
    gamma 5/3, rho 1, e 0, unit radial inflow.  nr=75, ntheta=30 is
    noh_small and nr=1800, ntheta=720 noh_large."""
    return f"""&CONTROL
 time_start=0.0
 time_end={time_end!r}
 dt_initial=1.0e-4
 dt_max=1.0e-2
 dt_min=1.0e-8
 dt_g=1.02
 cfl_sf=0.5
 cvisc1=0.5
 cvisc2=0.75
/
&EOS
 eos_type(1)='ideal gas'
 eos_param(1,1)=1.6666667
/
&CUTOFF
 zcut=1.0e-40
 accut=1.0e-40
 pcut=1.0e-40
/
&MESH
 region_typ(1)='LIN2'
 region_dim(1,:)={nr},{ntheta}
 region_material(1)=1
 region_side(1,1,:)=1,1
 region_side(1,2,:)=1,2
 region_side(1,3,:)=1,3
 region_side(1,4,:)=1,4
 segment_typ(:)='LINE','ARC_A','LINE','ARC_C'
 segment_bc(:)='SLIPY','FREE','SLIPX','WALL'
 segment_pos(1,:)=0.005,0.0,1.0,0.0
 segment_pos(2,:)=1.0,0.0,0.0,1.0,0.0,0.0
 segment_pos(3,:)=0.0,1.0,0.0,0.005
 segment_pos(4,:)=0.0,0.005,0.005,0.0,0.0,0.0
/
&INDICATORS
 region_type(1)='mesh'
 region_name(1)='air'
 material_type(1)='mesh'
 material_name(1)='air'
/
&INITIAL_CONDITIONS
 thermodynamic_type(1)='material'
 thermodynamic_value(1)=1
 density(1)=1.0
 energy(1)=0.0
 kinematic_type(1)='background'
 kinematic_value(1)=1
 kinematic_geometry(1)='radial'
 kinematic_param(1,1)=-1.0
 kinematic_param(2:3,1)=0.0
/
"""


def sod_multimaterial(nx=100, ny=25, time_end=20.0, vf=0.5):
    """Two-material Sod with mixed cells, the reference's sod_mm_lag_small
    set-up (material shape with a fixed volume fraction)."""
    return f"""&CONTROL
 time_start=0.0
 time_end={time_end!r}
 dt_initial=1.0e-3
 dt_max=1.0e-1
 dt_min=1.0e-8
 dt_g=1.02
 cfl_sf=0.5
 cvisc1=0.5
 cvisc2=0.75
/
&EOS
 eos_type(1)='ideal gas'
 eos_param(1,1)=1.4
 eos_type(2)='ideal gas'
 eos_param(1,2)=1.2
/
""" + _mesh(nx, ny, 0.0, 0.0, 100.0, 25.0, ("SLIPY", "SLIPX", "SLIPY", "SLIPX")) + f"""&INDICATORS
 region_type(1)='background'
 region_name(1)='shocktube'
 material_type(1)='background'
 material_name(1)='air'
 material_type(2)='shape'
 material_name(2)='helium'
 material_value(2)=1
/
&INITIAL_CONDITIONS
 thermodynamic_type(1)='region'
 thermodynamic_value(1)=1
 density(1)=1.0
 energy(1)=2.5
 thermodynamic_type(2)='material'
 thermodynamic_value(2)=2
 density(2)=0.125
 energy(2)=2.0
/
&SHAPES
 shape_type(1)='rectangle'
 shape_param(1,:)=50.5,-10.0,150.0,50.0,{vf!r}
/
"""


# The equations of state other than the ideal gas (eos_kn_forms.f90:28-106)
# in a two-material tube: material 2 of the given form fills one half, with
# a column of mixed cells (volume fraction vf) at the interface, material 1
# is an ideal gas.  Parameters (eos_param(1:6,2)): void -- the pressure;
# Tait -- B, gamma, rho0, the pressure floor (a water-like liquid, set
# slightly below rho0 so that the floor holds ahead of the shock);
# JWL -- omega, A, B, R1, R2, rho0 (TNT-like detonation products).
EOS_FORMS = {
    "void": ("VOID", (0.0,), "right", 0.01, 0.0),
    "tait": ("TAIT", (3.0, 7.15, 1.0, -0.1), "right", 0.99, 0.0),
    "jwl": ("JWL", (0.28, 3.712, 0.0323, 4.15, 0.95, 1.63), "left", 1.63, 1.0),
}


def eos_tube(form, nx=100, ny=10, time_end=20.0, vf=0.5):
    """Two-material tube on [0,100]x[0,10] whose material 2 uses the EoS
    form "void", "tait" or "jwl" (EOS_FORMS) over half of it; material 1 is
    air (gamma 1.4) at rho 1, e 2.5 (p 1) where material 2 sits on the
    right and at rho 0.125, e 2 (p 0.1) where it sits on the left."""
    name, params, side, rho2, e2 = EOS_FORMS[form]
    pl = "\n".join(" eos_param(%d,2)=%r" % (k + 1, v) for k, v in enumerate(params))
    rect = "50.5,-10.0,150.0,50.0" if side == "right" else "-50.0,-10.0,49.5,50.0"
    rho1, e1 = (1.0, 2.5) if side == "right" else (0.125, 2.0)
    return f"""&CONTROL
 time_start=0.0
 time_end={time_end!r}
 dt_initial=1.0e-3
 dt_max=1.0e-1
 dt_min=1.0e-8
 dt_g=1.02
 cfl_sf=0.5
 cvisc1=0.5
 cvisc2=0.75
/
&EOS
 eos_type(1)='ideal gas'
 eos_param(1,1)=1.4
 eos_type(2)='{name}'
{pl}
/
""" + _mesh(nx, ny, 0.0, 0.0, 100.0, 10.0, ("SLIPY", "SLIPX", "SLIPY", "SLIPX")) + f"""&INDICATORS
 region_type(1)='background'
 region_name(1)='tube'
 material_type(1)='background'
 material_name(1)='air'
 material_type(2)='shape'
 material_name(2)='{form}'
 material_value(2)=1
/
&INITIAL_CONDITIONS
 thermodynamic_type(1)='region'
 thermodynamic_value(1)=1
 density(1)={rho1!r}
 energy(1)={e1!r}
 thermodynamic_type(2)='material'
 thermodynamic_value(2)=2
 density(2)={rho2!r}
 energy(2)={e2!r}
/
&SHAPES
 shape_type(1)='rectangle'
 shape_param(1,:)={rect},{vf!r}
/
"""


def ensemble(n=512, seed=20240607, side_min=32, side_max=512):
    """Decks of a seeded ensemble of independent Eulerian problems: half Sod
    (gamma ~ U(1.2, 1.8), pressure ratio ~ logU(2, 1e4), density ratio 8,
    t = 0.2) and half Sedov (gamma ~ U(1.2, 1.8), t = 1.0), mesh side ~
    logU(side_min, side_max); a Sod tube of side s has about s^2 square
    cells (s*sqrt(10) x s/sqrt(10)).  Returns [(deck, meta)] with meta the
    drawn parameters."""
    import math
    import random
    rng = random.Random(seed)
    out = []
    for i in range(n):
        side = int(round(math.exp(rng.uniform(math.log(side_min), math.log(side_max)))))
        gamma = rng.uniform(1.2, 1.8)
        if i % 2 == 0:
            ratio = math.exp(rng.uniform(math.log(2.0), math.log(1.0e4)))
            nx = max(4, int(round(side * math.sqrt(10.0))))
            ny = max(2, int(round(side / math.sqrt(10.0))))
            deck = sod(nx, ny, time_end=0.2, eulerian=True, gamma=gamma, pratio=ratio)
            meta = {"kind": "sod", "side": side, "nx": nx, "ny": ny, "gamma": gamma,
                    "pratio": ratio}
        else:
            deck = sedov(side, time_end=1.0, eulerian=True, gamma=gamma)
            meta = {"kind": "sedov", "side": side, "nx": side, "ny": side, "gamma": gamma}
        out.append((deck, meta))
    return out


def sod_interface(nx=2000, ny=200, time_end=0.2, amplitude=0.02, periods=8, seed=7,
                  rho_right=0.125, p_right=0.1, tilt=0.0):
    """Two-material Sod tube on [0,1]x[0,0.1] with a sinusoidal interface
    x = 0.5 + amplitude*sin(2 pi periods y / 0.1 + phase) + tilt*(y - 0.05)
    (phase drawn from ``seed``): material 1 (gamma 1.4, rho 1, p 1) left of it, material 2
    (gamma 1.67, rho_right, p_right) right.  Returns (deck, fraction) where
    ``fraction(cnx, cny)`` gives each cell's area fraction of material 2
    (Gauss quadrature), for Problem.from_deck(deck, material_fraction=fraction)."""
    import math
    import random

    import numpy as np
    phase = random.Random(seed).uniform(0.0, 2.0 * math.pi)
    H = 0.1
    g2 = 1.67
    e1 = 2.5
    e2 = p_right / ((g2 - 1.0) * rho_right)
    deck = f"""&CONTROL
 time_start=0.0
 time_end={time_end!r}
 dt_initial=1.0e-5
 dt_max=1.0e-3
 dt_min=1.0e-10
 dt_g=1.02
 cfl_sf=0.5
 cvisc1=0.5
 cvisc2=0.75
/
&EOS
 eos_type(1)='ideal gas'
 eos_param(1,1)=1.4
 eos_type(2)='ideal gas'
 eos_param(1,2)={g2!r}
/
""" + _mesh(nx, ny, 0.0, 0.0, 1.0, H, ("SLIPY", "SLIPX", "SLIPY", "SLIPX")) + f"""&INDICATORS
 region_type(1)='background'
 region_name(1)='tube'
 material_type(1)='background'
 material_name(1)='left'
 material_type(2)='shape'
 material_name(2)='right'
 material_value(2)=1
/
&INITIAL_CONDITIONS
 thermodynamic_type(1)='region'
 thermodynamic_value(1)=1
 density(1)=1.0
 energy(1)={e1!r}
 thermodynamic_type(2)='material'
 thermodynamic_value(2)=2
 density(2)={rho_right!r}
 energy(2)={e2!r}
/
&SHAPES
 shape_type(1)='rectangle'
 shape_param(1,:)=2.0,2.0,3.0,3.0,1.0
/
"""

    def interface(y):
        return (0.5 + amplitude * np.sin(2.0 * np.pi * periods * y / H + phase) +
                tilt * (y - 0.5 * H))

    def fraction(cnx, cny):
        x0, x1 = cnx.min(axis=1), cnx.max(axis=1)
        y0, y1 = cny.min(axis=1), cny.max(axis=1)
        reach = abs(amplitude) + 0.5 * H * abs(tilt)
        vf = np.where(x0 >= 0.5 + reach, 1.0, 0.0)
        band = (x1 > 0.5 - reach) & (x0 < 0.5 + reach)
        if np.any(band):
            gx, gw = np.polynomial.legendre.leggauss(8)
            nsub = 64
            bx0, bx1, by0, by1 = x0[band], x1[band], y0[band], y1[band]
            h = (by1 - by0) / nsub
            acc = np.zeros(len(bx0))
            for k in range(nsub):
                a = by0 + k * h
                for xi, wi in zip(gx, gw):
                    y = a + 0.5 * h * (xi + 1.0)
                    wid = np.clip(bx1 - np.maximum(interface(y), bx0), 0.0, bx1 - bx0)
                    acc += 0.5 * h * wi * wid
            f = acc / ((bx1 - bx0) * (by1 - by0))
            f = np.where(f < 1e-12, 0.0, np.where(f > 1.0 - 1e-12, 1.0, f))
            vf[band] = f
        return vf

    return deck, fraction
