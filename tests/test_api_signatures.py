"""The drop-in surface: every public function of the path has the
reference's parameters, in the reference's order, with the reference's
defaults (tests/golden/ref_api.json, recorded by make_golden.py from the
reference's own functions with inspect.signature).  The package may add
keyword parameters after them (precision, device buffers).  A caller that
swaps the reference's import for this package's -- or registers these
functions in the reference's imaging_contexts() -- passes the same
arguments."""
import importlib
import inspect
import json
import os

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
SUBMODULES = ('imaging', 'gridding', 'kernels', 'weighting', 'coalesce', 'calibration', 'deconvolution',
              'skycomponents')

with open(os.path.join(HERE, 'golden', 'ref_api.json')) as f:
    RECORDS = json.load(f)


def _ours(arl, name):
    fn = getattr(arl, name, None)
    for sub in SUBMODULES:
        if fn is not None:
            break
        fn = getattr(importlib.import_module('algorithm-reference-library_gb300.' + sub), name, None)
    return fn


@pytest.mark.parametrize('rec', RECORDS, ids=[r['name'] for r in RECORDS])
def test_signature_matches_reference(arl, rec):
    fn = _ours(arl, rec['name'])
    assert fn is not None, '%s (%s) is not in the package' % (rec['name'], rec['module'])
    ours = list(inspect.signature(fn).parameters.values())
    index = {p.name: i for i, p in enumerate(ours)}
    for i, p in enumerate(rec['params']):
        if p['kind'] == 'VAR_KEYWORD':
            assert any(q.kind == inspect.Parameter.VAR_KEYWORD for q in ours), (rec['name'], '**kwargs')
            continue
        assert p['name'] in index, (rec['name'], 'missing parameter', p['name'])
        assert index[p['name']] == i, (rec['name'], p['name'], 'position', index[p['name']], i)
        q = ours[i]
        has = q.default is not inspect.Parameter.empty
        assert has == p['has_default'], (rec['name'], p['name'], 'default presence')
        literal = not (isinstance(p['default'], str) and p['default'].startswith('<') and p['default'].endswith('>'))
        if has and literal:
            assert q.default == p['default'], (rec['name'], p['name'], q.default, p['default'])
    # anything the package adds comes after the reference's parameters
    nref = len([p for p in rec['params'] if p['kind'] != 'VAR_KEYWORD'])
    for q in ours[nref:]:
        assert q.kind in (inspect.Parameter.KEYWORD_ONLY, inspect.Parameter.VAR_KEYWORD) or \
            q.default is not inspect.Parameter.empty, (rec['name'], 'added parameter without default', q.name)
