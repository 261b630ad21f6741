"""Small input models shared by the parity tests (each runs in well under a second)."""

BASE = """#domain: {dom}
#dx_dy_dz: 0.001 0.001 0.001
#time_window: {steps}
"""

MODELS = {
    # free space, default CFS PML (HORIPML order 1), z-dipole
    'fs_hori1': BASE.format(dom='0.030 0.030 0.030', steps=150) + """#pml_cells: 6
#waveform: ricker 1 1.5e9 w
#hertzian_dipole: z 0.015 0.015 0.015 w
#rx: 0.020 0.015 0.015
#rx: 0.012 0.018 0.011 r2 Ex Ey Ez Hx Hy Hz Ix Iy Iz
""",
    # PML off
    'pml_off': BASE.format(dom='0.024 0.022 0.020', steps=120) + """#pml_cells: 0
#waveform: gaussiandot 1 1e9 w
#hertzian_dipole: y 0.012 0.011 0.010 w
#rx: 0.016 0.011 0.010
""",
    # HORIPML order 2 with unequal slabs
    'hori2': BASE.format(dom='0.032 0.028 0.026', steps=140) + """#pml_cells: 5 4 6 6 5 4
#pml_cfs: constant forward 0 0 constant forward 1 1 sextic forward 0 0.5836
#pml_cfs: constant forward 0.05 0.05 cubic forward 1 8 quadratic forward 0 5.8357
#waveform: gaussiandotnorm 1 2e9 w
#hertzian_dipole: x 0.016 0.014 0.013 w
#rx: 0.020 0.016 0.012
""",
    # MRIPML order 1 and 2
    'mri1': BASE.format(dom='0.028 0.030 0.026', steps=130) + """#pml_cells: 6
#pml_formulation: MRIPML
#pml_cfs: constant forward 0.05 0.05 quartic forward 1 8 quartic forward 0 11.67
#waveform: ricker 1 2e9 w
#hertzian_dipole: z 0.014 0.015 0.013 w
#rx: 0.018 0.013 0.015
""",
    'mri2': BASE.format(dom='0.028 0.026 0.030', steps=130) + """#pml_cells: 5
#pml_formulation: MRIPML
#pml_cfs: constant forward 0 0 constant forward 1 1 sextic forward 0 0.5836
#pml_cfs: constant forward 0.05 0.05 cubic forward 1 8 quadratic forward 0 5.8357
#waveform: ricker 1 2e9 w
#hertzian_dipole: y 0.014 0.013 0.015 w
#rx: 0.010 0.016 0.017
""",
    # single-pole Debye block with smoothing at its faces
    'debye1': BASE.format(dom='0.030 0.028 0.026', steps=150) + """#pml_cells: 6
#material: 4.9 0.001 1 0 water
#add_dispersion_debye: 1 75.2 9.231e-12 water
#material: 6 0.002 1 0 sand
#box: 0.004 0.004 0.004 0.026 0.024 0.012 water
#sphere: 0.015 0.014 0.018 0.004 sand
#waveform: ricker 1 1.5e9 w
#hertzian_dipole: z 0.015 0.014 0.016 w
#rx: 0.019 0.014 0.016
""",
    # multi-pole Debye, Lorentz, Drude, all source kinds, anisotropic box, currents
    'mixed': BASE.format(dom='0.040 0.036 0.032', steps=100) + """#pml_cells: 6 5 4 5 6 4
#pml_formulation: MRIPML
#pml_cfs: constant forward 0 0 constant forward 1 1 sextic forward 0 0.5836
#pml_cfs: constant forward 0.05 0.05 cubic forward 1 8 quadratic forward 0 5.8357
#material: 4 0.01 1 0 half
#material: 6 0.001 1 0 soil
#material: 3 0 1 0 lor
#material: 2 0 1 0 dru
#material: 5 0 1 0 ax
#material: 7 0 1 0 ay
#material: 9 0 1 0 az
#add_dispersion_lorentz: 1 2.5 1e9 1e8 lor
#add_dispersion_drude: 1 1e9 1e8 0 dru
#add_dispersion_debye: 2 3 1e-9 2 1e-10 soil
#waveform: ricker 1 1.5e9 w
#waveform: gaussiandot 1 2e9 w2
#hertzian_dipole: z 0.020 0.018 0.016 w
#voltage_source: y 0.015 0.012 0.020 50 w2
#voltage_source: x 0.022 0.020 0.012 0 w 1e-11 5e-11
#magnetic_dipole: x 0.025 0.014 0.018 w2
#rx: 0.024 0.018 0.016
#rx: 0.010 0.010 0.010 r2 Ex Hz Ix Iy Iz
#box: 0 0 0 0.040 0.036 0.010 half
#sphere: 0.020 0.018 0.016 0.006 soil
#cylinder: 0.010 0.005 0.020 0.010 0.030 0.020 0.004 lor
#cylinder: 0.030 0.010 0.005 0.030 0.010 0.028 0.003 dru n
#box: 0.005 0.005 0.024 0.012 0.012 0.030 pec
#box: 0.026 0.024 0.020 0.034 0.030 0.028 ax ay az
#snapshot: 0.004 0.004 0.004 0.036 0.032 0.028 0.002 0.002 0.002 60 snap1
""",
    # 2D TMz (one cell in z): Debye block, z dipole, PML in x and y
    'tmz': BASE.format(dom='0.060 0.050 0.001', steps=160) + """#pml_cells: 8 8 0 8 8 0
#material: 5 0.002 1 0 soil
#add_dispersion_debye: 1 6 1e-9 soil
#box: 0 0 0 0.060 0.020 0.001 soil
#cylinder: 0.030 0.012 0 0.030 0.012 0.001 0.004 pec
#waveform: ricker 1 3e9 w
#hertzian_dipole: z 0.030 0.030 0 w
#rx: 0.036 0.030 0
#rx: 0.012 0.040 0 r2 Ez Hx Hy Ix Iy Iz
""",
    # 2D TMx (one cell in x): x dipole, unequal PML, a magnetic dipole
    'tmx': BASE.format(dom='0.001 0.044 0.052', steps=150) + """#pml_cells: 0 6 7 0 5 8
#material: 4 0.01 1 0 half
#box: 0 0 0 0.001 0.044 0.018 half
#waveform: gaussiandot 1 4e9 w
#hertzian_dipole: x 0 0.022 0.030 w
#rx: 0 0.030 0.030
#rx: 0 0.015 0.040 r2 Ex Hy Hz
""",
    # 2D TMy (one cell in y): y dipole, MRIPML order 2
    'tmy': BASE.format(dom='0.048 0.001 0.046', steps=150) + """#pml_cells: 6 0 5 7 0 6
#pml_formulation: MRIPML
#pml_cfs: constant forward 0 0 constant forward 1 1 sextic forward 0 0.5836
#pml_cfs: constant forward 0.05 0.05 cubic forward 1 8 quadratic forward 0 5.8357
#waveform: ricker 1 3e9 w
#hertzian_dipole: y 0.024 0 0.023 w
#rx: 0.030 0 0.023
""",
    # transmission lines (one with a delayed, shortened drive), a Debye half-space, a
    # Hertzian dipole and a voltage source alongside
    'tline': BASE.format(dom='0.036 0.034 0.040', steps=140) + """#pml_cells: 6
#material: 5 0.002 1 0 soil
#add_dispersion_debye: 1 6 1e-9 soil
#box: 0 0 0 0.036 0.034 0.014 soil
#waveform: gaussian 1 3e9 g
#waveform: ricker 1 4e9 r
#transmission_line: z 0.018 0.017 0.020 50 g
#transmission_line: x 0.012 0.022 0.026 73 r 2e-11 2e-10
#hertzian_dipole: y 0.024 0.012 0.022 r
#voltage_source: z 0.014 0.012 0.024 25 g
#rx: 0.022 0.017 0.020
#rx: 0.018 0.017 0.016 r2 Ez Hx Iz
""",
    # sources on the upper domain faces and a receiver on a face (boundary index paths)
    'faces': BASE.format(dom='0.020 0.018 0.016', steps=90) + """#pml_cells: 0
#waveform: gaussiandot 1 2e9 w
#hertzian_dipole: z 0.020 0.009 0.008 w
#hertzian_dipole: x 0.010 0.018 0.008 w
#voltage_source: y 0.010 0.009 0.016 0 w
#magnetic_dipole: z 0.010 0.009 0.016 w
#hertzian_dipole: z 0.010 0.009 0.008 w
#rx: 0.010 0.009 0.000
#rx: 0.011 0.010 0.009
""",
    # fractal soil from a Peplinski mixing model (no smoothing), a second box smoothed. The
    # mixing-model parameters are ones whose water-fraction powers come out the same through
    # numpy's vectorised pow and the C library's pow, so the material values do not depend
    # on the machine that builds the model.
    'fractal': BASE.format(dom='0.034 0.032 0.036', steps=120) + """#pml_cells: 6
#soil_peplinski: 0.5 0.5 2.0 2.66 0.001 0.3 soil
#soil_peplinski: 0.7 0.2 1.8 2.6 0.05 0.15 wet
#fractal_box: 0 0 0 0.034 0.032 0.016 1.5 1 1 1 8 soil lower 7
#fractal_box: 0.008 0.010 0.016 0.026 0.022 0.024 2.2 1 0.5 2 5 wet upper 3 y
#waveform: ricker 1 2e9 w
#hertzian_dipole: z 0.017 0.016 0.026 w
#rx: 0.021 0.016 0.026
#rx: 0.017 0.016 0.012 deep Ex Ey Ez Hx Hy Hz
""",
    # every geometry primitive, with and without smoothing: boxes (isotropic and anisotropic),
    # a sphere, oblique and axis-aligned cylinders, an edge, a plate, a resistive voltage source
    'smoothed': BASE.format(dom='0.024 0.022 0.020', steps=80) + """#pml_cells: 4
#material: 3 0.001 1 0 a
#material: 5 0.002 1.5 0.001 b
#material: 8 0 1 0 c
#box: 0.003 0.003 0.003 0.018 0.016 0.012 a
#sphere: 0.012 0.011 0.010 0.005 b
#cylinder: 0.004 0.010 0.004 0.020 0.010 0.016 0.003 c
#cylinder: 0.006 0.004 0.002 0.006 0.004 0.018 0.002 b n
#box: 0.014 0.002 0.014 0.020 0.008 0.019 a b c
#edge: 0.002 0.002 0.002 0.010 0.002 0.002 pec
#plate: 0.004 0.018 0.004 0.012 0.018 0.010 c
#waveform: ricker 1 2e9 w
#voltage_source: z 0.012 0.011 0.010 50 w
#hertzian_dipole: x 0.008 0.014 0.015 w
#rx: 0.010 0.010 0.010
#rx: 0.016 0.012 0.006 r2 Ex Ey Ez Hx Hy Hz
""",
    # a fractal soil box with rough top and x-minus faces and surface water on the top
    'rough': BASE.format(dom='0.040 0.036 0.040', steps=110) + """#pml_cells: 6
#soil_peplinski: 0.5 0.5 2.0 2.66 0.001 0.3 soil
#fractal_box: 0 0 0 0.040 0.036 0.020 1.5 1 1 1 8 soil box 7
#add_surface_roughness: 0 0 0.020 0.040 0.036 0.020 1.5 1 1 0.015 0.025 box 12
#add_surface_water: 0 0 0.020 0.040 0.036 0.020 0.022 box
#add_surface_roughness: 0 0 0 0 0.036 0.020 1.8 1 1 0 0.006 box 5
#waveform: ricker 1 2e9 w
#hertzian_dipole: z 0.020 0.018 0.030 w
#rx: 0.024 0.018 0.030
#rx: 0.020 0.018 0.021 wet Ex Ey Ez Hx Hy Hz
""",
    # a receiver array (4 x 3 x 1, zero step along z) after a single receiver
    'rxarray': """#title: receiver array
#domain: 0.030 0.028 0.026
#dx_dy_dz: 0.001 0.001 0.001
#time_window: 80
#pml_cells: 5
#material: 4 0.001 1 0 block
#box: 0.010 0.008 0.006 0.020 0.020 0.014 block
#waveform: gaussiandot 1 3e9 w
#hertzian_dipole: y 0.015 0.014 0.018 w
#rx: 0.012 0.014 0.018
#rx_array: 0.008 0.010 0.012 0.022 0.016 0.012 0.004 0.003 0
""",
    # triangles on all three grid planes: zero-thickness PEC faces, prisms with and without
    # smoothing, a uniaxial prism of three materials, vertices in both windings
    'triangles': """#title: triangles
#domain: 0.040 0.036 0.032
#dx_dy_dz: 0.001 0.001 0.001
#time_window: 90
#pml_cells: 5
#material: 4 0.001 1 0 d1
#material: 7 0.002 1 0 d2
#material: 2.5 0 1 0 d3
#triangle: 0.008 0.008 0.006 0.020 0.010 0.006 0.012 0.024 0.006 0 pec
#triangle: 0.030 0.006 0.010 0.030 0.026 0.014 0.030 0.012 0.026 0.004 d1
#triangle: 0.006 0.028 0.008 0.024 0.028 0.024 0.010 0.028 0.026 0.003 d2 n
#triangle: 0.014 0.006 0.020 0.033 0.018 0.020 0.016 0.030 0.020 0.002 d1 d2 d3
#triangle: 0.022 0.012 0.006 0.022 0.022 0.016 0.022 0.008 0.018 0 pec
#waveform: gaussiandot 1 4e9 w
#hertzian_dipole: z 0.018 0.017 0.016 w
#rx: 0.021 0.015 0.014
#rx: 0.026 0.020 0.022 r2 Ex Ey Ez Hx Hy Hz
""",
    # cylindrical sectors on all three planes: a zero-thickness PEC sector, prisms with and
    # without smoothing, a uniaxial prism, a sector crossing the 0/360 degree line and one
    # clipped by the domain
    'sectors': """#title: cylindrical sectors
#domain: 0.040 0.036 0.032
#dx_dy_dz: 0.001 0.001 0.001
#time_window: 90
#pml_cells: 5
#material: 4 0.001 1 0 d1
#material: 7 0.002 1 0 d2
#material: 2.5 0 1 0 d3
#cylindrical_sector: z 0.014 0.012 0.006 0.006 0.008 20 110 pec
#cylindrical_sector: x 0.018 0.016 0.026 0.030 0.009 300 120 d1
#cylindrical_sector: y 0.010 0.010 0.024 0.028 0.007 45 270 d2 n
#cylindrical_sector: z 0.026 0.024 0.018 0.021 0.010 90 200 d1 d2 d3
#cylindrical_sector: x 0.034 0.004 0.012 0.016 0.006 0 90 d3
#cylindrical_sector: z 0.038 0.030 0.010 0.014 0.005 180 150 d2
#waveform: gaussiandot 1 4e9 w
#hertzian_dipole: z 0.020 0.019 0.015 w
#rx: 0.023 0.017 0.013
#rx: 0.026 0.022 0.022 r2 Ex Ey Ez Hx Hy Hz
""",
}


def build_fixture(g, **kw):
    """The grid of a golden fixture: its input text through the front-end (with the files it
    reads, such as an excitation file, written beside it first) and, for a B-scan fixture, the
    recorded model run in the namespace of its #python blocks and its sources and receivers
    stepped to that run."""
    import os
    import tempfile
    from gprmax_gb300.model import build_grid, step_sources_receivers
    from gprmax_gb300.constants import c, e0, m0, z0
    files = {k[len('file_'):]: str(v) for k, v in g.items() if k.startswith('file_')}
    with tempfile.TemporaryDirectory() as tmp:
        for name, text in files.items():
            with open(os.path.join(tmp, name), 'w') as f:
                f.write(text)
        inputfile = os.path.join(tmp, 'model.in') if files else ''
        namespace = None
        if 'model_run' in g:   # what #python blocks see for that model run
            namespace = {'c': c, 'e0': e0, 'm0': m0, 'z0': z0,
                         'number_model_runs': int(g['model_end']),
                         'current_model_run': int(g['model_run']),
                         'inputfile': os.path.abspath(inputfile) if inputfile else ''}
        G = build_grid(str(g['input']).splitlines(True), messages=False, usernamespace=namespace,
                       inputfilename=inputfile, **kw)
    if 'model_run' in g:
        step_sources_receivers(G, int(g['model_run']), int(g['model_end']))
    return G
