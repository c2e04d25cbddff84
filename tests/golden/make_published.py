"""Collects the numbers pmwd itself published for seeded runs into
``published_pmwd.json`` (read by the tests; the reference tree is not
present where the GPU tests run).

    python tests/golden/make_published.py [path-to-pmwd-checkout]

Sources, all outputs printed by pmwd on an NVIDIA H100 PCIe:

* ``docs/papers/adjoint/grads.txt`` -- the cosmology gradients of 64
  repeated adjoint runs and 64 repeated automatic-differentiation runs of
  ``docs/papers/adjoint/grads.py`` (128^3 particles, mesh_shape 2, spacing
  1 Mpc/h, a_start 1/16, a_nbody_maxstep 1/16, SimpleLCDM; target density
  from white_noise(0), real modes from white_noise(1); objective
  var(density - target));
* ``docs/examples/quickstart.ipynb`` -- 256^3 particles, mesh_shape 2,
  spacing 1: the standard deviations of disp and vel after 2LPT (cell 14)
  and after the N-body run (cell 16) for white_noise(0) with A_s_1e9 2,
  n_s 0.96, Omega_m 0.3, Omega_b 0.05, h 0.7, and the cosmology gradients
  of the same objective as above with SimpleLCDM (cell 31).  The notebook
  prints 3 decimals.
* ``docs/examples/adjoint.ipynb`` -- the single-precision rows of its
  reproducibility table (cell 5: two identical forward runs to a = 1) and
  reversibility table (cell 11: forward to a = 1, then reverse=True back to
  a_start), 384^3 particles, white_noise(0), SimpleLCDM, for ptcl_spacing
  0.5 / 1, mesh_shape 2 / 1 and a_nbody_maxstep 1/64 / 1/128.  Each row
  prints the mesh cells per particle, the particle mass in 1e10 M_sun/h,
  the step count, the relative differences of disp and vel, and the
  standard deviations of disp and vel (after the N-body run in cell 5, of
  the 2LPT state in cell 11), 2 significant digits each.
"""

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
NAMES = ('A_s_1e9', 'n_s', 'Omega_m', 'Omega_b', 'h')


def cosmo_blocks(text):
    out = []
    for block in re.findall(r'Cosmology\((.*?)\)\s*$', text, flags=re.S | re.M):
        vals = {k: float(v) for k, v in re.findall(r'(\w+)=Array\(([-0-9.e]+)', block)}
        out.append([vals[k] for k in NAMES])
    return out


def outputs(cell):
    txt = []
    for o in cell.get('outputs', []):
        if 'text' in o:
            txt.append(''.join(o['text']))
        elif 'data' in o and 'text/plain' in o['data']:
            txt.append(''.join(o['data']['text/plain']))
    return '\n'.join(txt)


def notebook_rows(cell):
    """(ptcl_spacing, mesh_shape, a_nbody_maxstep) of each check_* call of a
    cell, zipped with its printed line."""
    src = ''.join(cell['source'])
    calls = re.findall(r"ptcl_spacing=([0-9.]+), mesh_shape=(\d+), a_nbody_maxstep=1/(\d+), "
                       r"float_dtype='(f[48])'", src)
    lines = [l for l in outputs(cell).splitlines() if l.strip()]
    assert len(calls) == len(lines) == 8
    rows = []
    for (sp, ms, inv, dt), line in zip(calls, lines):
        m = re.match(r'(f[48]), (\d+), (\d+), +(\d+): ([-0-9.e+]+), ([-0-9.e+]+); '
                     r'([-0-9.e+]+), ([-0-9.e+]+)$', line.strip())
        assert m and m.group(1) == dt, line
        rows.append({'ptcl_spacing': float(sp), 'mesh_shape': int(ms),
                     'a_nbody_maxstep_inv': int(inv), 'cells_per_ptcl': int(m.group(2)),
                     'ptcl_mass_1e10': int(m.group(3)), 'steps': int(m.group(4)),
                     'disp_rel_diff': float(m.group(5)), 'vel_rel_diff': float(m.group(6)),
                     'disp_std': float(m.group(7)), 'vel_std': float(m.group(8))})
    return rows


def adjoint_notebook(root):
    nb = json.load(open(os.path.join(root, 'docs/examples/adjoint.ipynb')))
    cells = nb['cells']
    f4 = [c for c in cells if c['cell_type'] == 'code' and "float_dtype='f4')" in
          ''.join(c['source']) and 'check_' in ''.join(c['source'])
          and 'def ' not in ''.join(c['source'])]
    repro = [c for c in f4 if 'check_reproducibility(' in ''.join(c['source'])]
    rev = [c for c in f4 if 'check_reversibility(' in ''.join(c['source'])]
    assert len(repro) == len(rev) == 1
    return {'config': {'ptcl_grid_shape': [384, 384, 384], 'seed': 0, 'cosmo': 'SimpleLCDM',
                       'float_dtype': 'f4', 'digits': 2},
            'reproducibility': notebook_rows(repro[0]),
            'reversibility': notebook_rows(rev[0])}


def main(root):
    grads = open(os.path.join(root, 'docs/papers/adjoint/grads.txt')).read()
    adj, ad = grads.split('#### AD ####')
    nb = json.load(open(os.path.join(root, 'docs/examples/quickstart.ipynb')))
    cells = [c for c in nb['cells'] if c['cell_type'] == 'code']
    pairs = []
    for c in cells:
        m = re.search(r'\(Array\(([-0-9.]+), dtype=float32\), Array\(([-0-9.]+), dtype=float32\)\)',
                      outputs(c))
        if m:
            pairs.append([float(m.group(1)), float(m.group(2))])
    grad = [cosmo_blocks(outputs(c)) for c in cells if 'A_s_1e9=Array(51' in outputs(c)]
    out = {
        'names': list(NAMES),
        'grads_txt': {
            'config': {'ptcl_spacing': 1.0, 'ptcl_grid_shape': [128, 128, 128], 'mesh_shape': 2,
                       'a_start': 1 / 16, 'a_nbody_maxstep': 1 / 16, 'cosmo': 'SimpleLCDM',
                       'target_seed': 0, 'modes_seed': 1},
            'adjoint': cosmo_blocks(adj),
            'ad': cosmo_blocks(ad),
        },
        'quickstart': {
            'config': {'ptcl_spacing': 1.0, 'ptcl_grid_shape': [256, 256, 256], 'mesh_shape': 2},
            'cosmo': {'A_s_1e9': 2.0, 'n_s': 0.96, 'Omega_m': 0.3, 'Omega_b': 0.05, 'h': 0.7},
            'lpt_disp_vel_std': pairs[0],
            'nbody_disp_vel_std': pairs[1],
            'cosmo_grad': grad[0][0],
            'decimals': 3,
        },
    }
    out['adjoint_notebook'] = adjoint_notebook(root)
    assert len(out['grads_txt']['adjoint']) == 64 and len(out['grads_txt']['ad']) == 64
    with open(os.path.join(HERE, 'published_pmwd.json'), 'w') as f:
        json.dump(out, f, indent=1)
        f.write('\n')


if __name__ == '__main__':
    main(sys.argv[1] if len(sys.argv) > 1 else '/root/reference')
