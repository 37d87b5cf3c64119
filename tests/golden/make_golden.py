"""Generate the golden fixtures under tests/golden/ from the reference itself.

Run once in a container where the reference checkout is available:

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py <reference checkout> [main] [grads] [jtfs]

It imports the reference's numpy frontends (the ``kymatio.numpy`` namespace
is avoided because it pulls in the 3-D filter bank, whose scipy import fails
on current scipy) and writes:

* ``ref_test_data_2d.npz`` / ``ref_test_data_1d.npz`` -- the reference's own
  golden vectors (tests/scattering2d/test_data_2d.npz,
  tests/scattering1d/test_data_1d.npz) re-exported unchanged;
* ``ref_cases_2d.npz`` -- seeded inputs and reference numpy FP64 outputs for
  small 2-D configurations (odd, non-square, pre_pad, max_order=1, L=4, the
  256x256 J=3 shape);
* ``ref_cases_1d.npz`` -- the same for 1-D configurations (T local, global,
  zero, stride, the 8192-sample J=6 Q=(8,1) T=64 shape);
* ``ref_bank_2d.npz`` -- the full 40x40 J=2 filter bank and per-filter
  checksums of the 272x272 J=3 bank;
* ``ref_grads.npz`` -- input gradients from the reference torch frontend's
  autograd in float64 (x, upstream gradient g, d<g, S(x)>/dx) for 2-D and 1-D
  configurations;
* ``ref_jtfs.npz`` -- seeded inputs and reference numpy FP64 outputs of joint
  time-frequency scattering (formats 'time' and 'joint', out_type array, list
  and dict, F local / zero / global, T global), with each configuration's
  ``meta()`` (keys, n, order, n_fr, spin, time and frequential xi / sigma /
  j) and, for
  the array outputs, an upstream gradient and the reference torch frontend's
  float64 input gradient.

Nothing at test time reads the reference; the tests read these files.
"""
import io
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

CASES_2D = [
    # name, J, (M, N), L, max_order, pre_pad, batch
    ('j2_32', 2, (32, 32), 8, 2, False, 3),
    ('j1_31', 1, (31, 31), 8, 2, False, 2),
    ('j4_33', 4, (33, 33), 8, 2, False, 2),
    ('j5_37x32', 5, (37, 32), 8, 2, False, 2),
    ('j3_64x48', 3, (64, 48), 8, 2, False, 2),
    ('j2_20x24_prepad', 2, (20, 24), 8, 2, True, 2),
    ('j3_40_order1', 3, (40, 40), 8, 1, False, 2),
    ('j2_24_L4', 2, (24, 24), 4, 2, False, 2),
    ('j2_8', 2, (8, 8), 8, 2, False, 2),
    ('j3_256', 3, (256, 256), 8, 2, False, 1),
]

CASES_1D = [
    # name, kwargs, batch
    ('j6_q8_t64_n8192', dict(J=6, shape=8192, Q=(8, 1), T=64), 2),
    ('j4_q2_global_n300', dict(J=4, shape=300, Q=2, T='global'), 2),
    ('j5_q4_t0_n1024', dict(J=5, shape=1024, Q=4, T=0, out_type='list'), 2),
    ('j5_q3_stride4_n1000', dict(J=5, shape=1000, Q=3, stride=4), 2),
    ('j6_q8_os1_n512', dict(J=6, shape=512, Q=8, oversampling=1), 2),
    ('j3_q1_t8_n64_order1', dict(J=3, shape=64, Q=1, T=8, max_order=1), 3),
]


def main(ref_root):
    sys.path.insert(0, ref_root)
    from kymatio.scattering2d.frontend.numpy_frontend import ScatteringNumPy2D
    from kymatio.scattering1d.frontend.numpy_frontend import ScatteringNumPy1D

    for src, dst in [('tests/scattering2d/test_data_2d.npz', 'ref_test_data_2d.npz'),
                     ('tests/scattering1d/test_data_1d.npz', 'ref_test_data_1d.npz')]:
        with open(os.path.join(ref_root, src), 'rb') as f:
            data = np.load(io.BytesIO(f.read()))
            np.savez_compressed(os.path.join(HERE, dst), **{k: data[k] for k in data.files})

    out, meta = {}, []
    for i, (name, J, shape, L, mo, pp, B) in enumerate(CASES_2D):
        S = ScatteringNumPy2D(J, shape, L=L, max_order=mo, pre_pad=pp)
        xs = (B, S._M_padded, S._N_padded) if pp else (B,) + shape
        x = np.random.default_rng(100 + i).random(xs).astype(np.float32)
        y = S(x.astype(np.float64))
        out[name + '/x'] = x
        out[name + '/S'] = y.astype(np.float32) if name == 'j3_256' else y
        meta.append(dict(name=name, J=J, shape=list(shape), L=L, max_order=mo, pre_pad=pp))
    out['meta'] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, 'ref_cases_2d.npz'), **out)

    out, meta = {}, []
    for i, (name, kw, B) in enumerate(CASES_1D):
        S = ScatteringNumPy1D(**kw)
        x = np.random.default_rng(200 + i).standard_normal((B, kw['shape'])).astype(np.float32)
        y = S(x.astype(np.float64))
        out[name + '/x'] = x
        if isinstance(y, list):
            for p in y:
                out[name + '/S/' + ','.join(map(str, p['n']))] = p['coef']
        else:
            out[name + '/S'] = y
        meta.append(dict(name=name, kwargs=kw))
    out['meta'] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, 'ref_cases_1d.npz'), **out)

    from kymatio.scattering2d.filter_bank import filter_bank
    bank = filter_bank(40, 40, 2, 8)
    out = {}
    for r, lv in enumerate(bank['phi']['levels']):
        out['phi/%d' % r] = lv
    for n, p in enumerate(bank['psi']):
        for r, lv in enumerate(p['levels']):
            out['psi/%d/%d' % (n, r)] = lv
    big = filter_bank(272, 272, 3, 8)
    sums = []
    for lv in big['phi']['levels']:
        sums.append([lv.sum(dtype=np.float64), (lv.astype(np.float64) ** 2).sum(), lv[0, 0], lv[3, 5]])
    for p in big['psi']:
        for lv in p['levels']:
            sums.append([lv.sum(dtype=np.float64), (lv.astype(np.float64) ** 2).sum(), lv[0, 0], lv[3, 5]])
    out['big272/checksums'] = np.array(sums)
    np.savez_compressed(os.path.join(HERE, 'ref_bank_2d.npz'), **out)


GRAD_2D = [
    # name, J, (M, N), max_order, pre_pad, batch
    ('g2_j2_32', 2, (32, 32), 2, False, 2),
    ('g2_j4_128', 4, (128, 128), 2, False, 1),
    ('g2_j3_64x48', 3, (64, 48), 2, False, 1),
    ('g2_j1_31_prepad', 1, (31, 31), 2, True, 2),
    ('g2_j3_40_order1', 3, (40, 40), 1, False, 2),
    ('g2_j3_256', 3, (256, 256), 2, False, 1),
]
GRAD_1D = [
    ('g1_j5_q4_n1024', dict(J=5, shape=1024, Q=4), 2),
    ('g1_j6_q8_t64_n8192', dict(J=6, shape=8192, Q=(8, 1), T=64), 1),
]


def grads(ref_root):
    sys.path.insert(0, ref_root)
    import torch
    from kymatio.scattering2d.frontend.torch_frontend import ScatteringTorch2D
    from kymatio.scattering1d.frontend.torch_frontend import ScatteringTorch1D
    torch.set_num_threads(os.cpu_count() or 1)
    out = {}
    for i, (name, J, shape, mo, pp, B) in enumerate(GRAD_2D):
        S = ScatteringTorch2D(J, shape, max_order=mo, pre_pad=pp).double()
        xs = (B, S._M_padded, S._N_padded) if pp else (B,) + shape
        rng = np.random.default_rng(300 + i)
        x = rng.random(xs).astype(np.float32)
        xt = torch.from_numpy(x.astype(np.float64)).requires_grad_()
        y = S(xt)
        g = rng.standard_normal(tuple(y.shape)).astype(np.float32)
        y.backward(torch.from_numpy(g.astype(np.float64)))
        out[name + '/x'], out[name + '/g'], out[name + '/gx'] = x, g, xt.grad.numpy()
    for i, (name, kw, B) in enumerate(GRAD_1D):
        S = ScatteringTorch1D(**kw).double()
        rng = np.random.default_rng(400 + i)
        x = rng.standard_normal((B, kw['shape'])).astype(np.float32)
        xt = torch.from_numpy(x.astype(np.float64)).requires_grad_()
        y = S(xt)
        g = rng.standard_normal(tuple(y.shape)).astype(np.float32)
        y.backward(torch.from_numpy(g.astype(np.float64)))
        out[name + '/x'], out[name + '/g'], out[name + '/gx'] = x, g, xt.grad.numpy()
    meta = dict(g2=[dict(name=c[0], J=c[1], shape=list(c[2]), max_order=c[3], pre_pad=c[4]) for c in GRAD_2D],
                g1=[dict(name=c[0], kwargs=c[1]) for c in GRAD_1D])
    out['meta'] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, 'ref_grads.npz'), **out)


CASES_JTFS = [
    # name, kwargs, batch
    ('time_j6_jfr2_q82', dict(J=6, J_fr=2, Q=(8, 2), shape=1024, format='time'), 2),
    ('joint_j6_jfr2_q82', dict(J=6, J_fr=2, Q=(8, 2), shape=1024, format='joint'), 2),
    ('time_j5_jfr3_q41_F0_list', dict(J=5, J_fr=3, Q=(4, 1), shape=512, F=0, out_type='list', format='time'), 2),
    ('time_j5_jfr2_q4_global', dict(J=5, J_fr=2, Q=4, shape=512, T='global', F='global', format='time'), 2),
    ('joint_j5_jfr2_q41_dict', dict(J=5, J_fr=2, Q=(4, 1), shape=512, out_type='dict', format='joint'), 2),
    ('joint_j4_jfr1_q21_n300', dict(J=4, J_fr=1, Q=(2, 1), shape=300, format='joint'), 3),
]


def meta_n_json(n):
    """meta['n'] rows as JSON: a range as its list, NaN as null, an index as int."""
    def one(v):
        if isinstance(v, range):
            return list(v)
        if isinstance(v, float) and v != v:
            return None
        return int(v)
    return [[one(v) for v in row] for row in n]


def jtfs(ref_root):
    sys.path.insert(0, ref_root)
    from kymatio.scattering1d.frontend.numpy_frontend import TimeFrequencyScatteringNumPy
    out, meta = {}, []
    for i, (name, kw, B) in enumerate(CASES_JTFS):
        S = TimeFrequencyScatteringNumPy(**kw)
        x = np.random.default_rng(300 + i).standard_normal((B, kw['shape'])).astype(np.float32)
        y = S(x.astype(np.float64))
        out[name + '/x'] = x
        if isinstance(y, list):
            for p in y:
                out[name + '/S/' + ','.join(map(str, p['n']))] = p['coef']
        elif isinstance(y, dict):
            for k, v in y.items():
                out[name + '/S/' + ','.join(map(str, k))] = v
        else:
            out[name + '/S'] = y
        if not isinstance(y, (list, dict)):
            # input gradient through the reference torch frontend's autograd, float64
            import torch
            from kymatio.scattering1d.frontend.torch_frontend import TimeFrequencyScatteringTorch
            St = TimeFrequencyScatteringTorch(**kw).double()
            xt = torch.from_numpy(x.astype(np.float64)).requires_grad_()
            yt = St(xt)
            g = np.random.default_rng(350 + i).standard_normal(tuple(yt.shape)).astype(np.float32)
            yt.backward(torch.from_numpy(g.astype(np.float64)))
            out[name + '/g'], out[name + '/gx'] = g, xt.grad.numpy()
        m = S.meta()
        out[name + '/meta/key'] = np.array(json.dumps([list(map(int, k)) for k in m['key']]))
        out[name + '/meta/n'] = np.array(json.dumps(meta_n_json(m['n'])))
        for field in ('order', 'n_fr', 'spin', 'xi_fr', 'sigma_fr', 'j_fr', 'xi', 'sigma', 'j'):
            out[name + '/meta/' + field] = np.asarray(m[field], dtype=np.float64)
        meta.append(dict(name=name, kwargs=kw))
    out['meta'] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, 'ref_jtfs.npz'), **out)


if __name__ == '__main__':
    if len(sys.argv) < 2:
        sys.exit('usage: make_golden.py <reference checkout> [main] [grads] [jtfs]')
    root = sys.argv[1]
    what = sys.argv[2:] or ['main', 'grads', 'jtfs']
    if 'main' in what:
        main(root)
    if 'grads' in what:
        grads(root)
    if 'jtfs' in what:
        jtfs(root)
