"""Generate the golden fixtures that pin the CPU oracle (run in the build container).

Sources, all inside the reference µSpectre tree (read as text or imported, never
copied into this repository):

* ``tests/test_material_hyper_elasto_plastic1.cc:85-339`` -- HyperElastoPlastic1
  known answers (τ, bₑ, εₚ and the 9×9 tangent after an elastic and a plastic step),
  parsed from the ``<<`` initialiser lists of the C++ test.
* ``tests/header_test_eigen_tools.cc:42-62`` -- expm known answer.
* ``tests/test_fft_utils.cc:43-84`` -- fftfreq known answers.
* ``tests/python_goose_ref.py`` -- the GooseFFT NumPy projection used by
  ``tests/python_projection_tests.py:62-130``; imported here (with ``np.float`` mapped
  to ``float`` so that it runs on NumPy 2) to write Ĝ and projection results at 5² and
  5³ for the small- and finite-strain operators.

Usage:  python tests/golden/make_golden.py <path of the reference source tree>
Writes ``tests/golden/hep1_kat.json``, ``expm_kat.json``, ``fftfreq_kat.json`` and
``goose_projection.npz`` next to this script.
"""
import itertools
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _numbers(block):
    block = block.replace('pi', '__PI__')
    vals = []
    for tok in re.split(r'[,\s]+', block.strip()):
        if not tok:
            continue
        if '__PI__' in tok:
            coef = tok.replace('*__PI__', '').replace('__PI__', '1')
            vals.append(float(coef) * np.pi)
        else:
            vals.append(float(tok))
    return vals


def parse_hep1(ref):
    src = open(os.path.join(ref, 'tests/test_material_hyper_elasto_plastic1.cc')).read()
    # material constants of the fixture (lines 49-62)
    consts = {k: float(v) for k, v in re.findall(r'constexpr static Real (K|mu|H|tau_y0)\{([-+.\deE]+)\}', src)}
    blocks = [(name, _numbers(body)) for name, body in
              re.findall(r'(tau_ref|be_ref|C4_ref) <<(.*?);', src, flags=re.S)]
    eps = [float(v) for v in re.findall(r'Real ep_ref\{([-+.\deE]+)\}', src)]
    F01 = [float(v) for v in re.findall(r'F\(0, 1\) = ([-+.\deE]+);', src)]
    # test_evaluate_stiffness holds the complete sequence: elastic (τ, bₑ, C4) then
    # plastic (τ, bₑ, C4); its blocks come after the 4 blocks of test_evaluate_stress
    stiff = blocks[4:]
    names = [b[0] for b in stiff]
    assert names == ['tau_ref', 'be_ref', 'C4_ref', 'tau_ref', 'be_ref', 'C4_ref'], names
    steps = []
    for s in range(2):
        tau, be, C4 = (stiff[3 * s + i][1] for i in range(3))
        steps.append({'F01': F01[s], 'tau': np.array(tau).reshape(3, 3).tolist(),
                      'be': np.array(be).reshape(3, 3).tolist(), 'eps_p': eps[s],
                      'C4_rows': np.array(C4).reshape(9, 9).tolist()})
    return {'source': 'tests/test_material_hyper_elasto_plastic1.cc:49-339',
            'tol': 1e-8, 'K': consts['K'], 'mu': consts['mu'], 'H': consts['H'],
            'tau_y0': consts['tau_y0'], 'steps': steps}


def parse_expm(ref):
    src = open(os.path.join(ref, 'tests/header_test_eigen_tools.cc')).read()
    inp, out = re.findall(r'(?:input|output) <<(.*?);', src, flags=re.S)[:2]
    return {'source': 'tests/header_test_eigen_tools.cc:42-62', 'tol': 1e-8,
            'input': np.array(_numbers(inp)).reshape(3, 3).tolist(),
            'output': np.array(_numbers(out)).reshape(3, 3).tolist()}


def parse_fftfreq(ref):
    src = open(os.path.join(ref, 'tests/test_fft_utils.cc')).read()
    refs = [_numbers(b) for b in re.findall(r'ref\{(.*?)\};', src, flags=re.S)]
    return {'source': 'tests/test_fft_utils.cc:43-84',
            'cases': [{'n': 12, 'length': 1.0, 'freqs': refs[0]},
                      {'n': 10, 'length': 10.0, 'freqs': refs[1]}],
            'xi_cases': [{'res': [12, 10], 'lengths': [1.0, 10.0], 'ccoord': [2, 3], 'xi': [2.0, 0.3]},
                         {'res': [12, 10], 'lengths': [1.0, 10.0], 'ccoord': [7, 8], 'xi': [-5.0, -0.2]}]}


def goose_projection(ref):
    sys.path.insert(0, os.path.join(ref, 'tests'))
    if not hasattr(np, 'float'):
        np.float = float  # the GooseFFT script predates NumPy 2
    import python_goose_ref as g
    out = {}
    for ndim in (2, 3):
        for kind, cls in (('small', g.SmallStrainProjectionGooseFFT),
                          ('finite', g.FiniteStrainProjectionGooseFFT)):
            # python_projection_tests.py:126-130: (ndim, 5, 2, 70e9, .33, 3.)
            gref = cls(ndim, 5, 2, 70e9, .33, 3.)
            shape = [5] * ndim
            strain_shape = (ndim, ndim, *shape)
            strain = np.arange(np.prod(strain_shape)).reshape(strain_shape).astype(float)
            if kind == 'small':
                strain += strain.transpose(1, 0, *range(2, len(strain.shape)))
            b_g = gref.G(strain.copy()).reshape(strain.shape)
            key = '%s_%dd' % (kind, ndim)
            out[key + '_strain'] = strain
            out[key + '_result'] = b_g
            out[key + '_ghat4'] = gref.Ghat4
    return out


def main(ref):
    with open(os.path.join(HERE, 'hep1_kat.json'), 'w') as f:
        json.dump(parse_hep1(ref), f, indent=1)
    with open(os.path.join(HERE, 'expm_kat.json'), 'w') as f:
        json.dump(parse_expm(ref), f, indent=1)
    with open(os.path.join(HERE, 'fftfreq_kat.json'), 'w') as f:
        json.dump(parse_fftfreq(ref), f, indent=1)
    np.savez_compressed(os.path.join(HERE, 'goose_projection.npz'), **goose_projection(ref))


if __name__ == '__main__':
    if len(sys.argv) != 2:
        sys.exit('usage: make_golden.py <path of the reference source tree>')
    main(sys.argv[1])
