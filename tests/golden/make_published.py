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
    assert len(out['grads_txt']['adjoint']) == 64 and len(out['grads_txt']['ad']) == 64
    with open(os.path.join(HERE, 'published_pmwd.json'), 'w') as f:
        json.dump(out, f, indent=1)
        f.write('\n')


if __name__ == '__main__':
    main(sys.argv[1] if len(sys.argv) > 1 else '/root/reference')
