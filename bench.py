"""Throughput of the scattering hot path on GB300 (one JSON line on rank 0).

Workload: Scattering2D J=3, L=8, max_order=2 on 256x256 float32 Gaussian
random fields (white N(0,1) smoothed by an isotropic Gaussian of sigma
U[1,4] px, rescaled to [0,1]; seed 2), batch 64 per GPU.  One step = one
forward over the batch.  Inputs are generated synthetically (no dataset).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
  python bench.py --extra NAME      # one of the other workloads alone (profiling)

--impl reference times the reference's own CPU implementation of the path:
kymatio's stock ``ScatteringTorch2D`` (torch on the host cores, float32, all
host threads), pip-installed from the reference into baseline/_ref, on the
full 64-image batch per step.  Where that install is missing it falls back to
the oracle port of kymatio's numpy backend (``kind: "port"``).
Under torchrun each rank is an independent replica (images shard with no
exchange step): value = images over all ranks / max time over ranks.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

J, L, SIDE = 3, 8, 256
BATCH = 64
METRIC = 'Scattering2D 256^2 J=3 L=8 img/s'


def grf_batch(n, seed=2, side=SIDE):
    """Gaussian random fields rescaled to [0,1] (float32)."""
    from scipy.ndimage import gaussian_filter
    rng = np.random.default_rng(seed)
    out = np.empty((n, side, side), np.float32)
    for i in range(n):
        w = rng.standard_normal((side, side))
        s = rng.uniform(1.0, 4.0)
        g = gaussian_filter(w, s, mode='wrap')
        g = (g - g.min()) / (g.max() - g.min())
        out[i] = g.astype(np.float32)
    return out


def algorithmic_bytes_per_image(J=J, L=L, side=SIDE):
    """Compulsory HBM bytes of the plain path per image: input, output and one
    write + one read of every order-1 parent spectrum (fp32 complex)."""
    Mp = ((side + 2 ** J) // 2 ** J + 1) * 2 ** J
    C = 1 + J * L + L * L * J * (J - 1) // 2
    out = 4 * C * (side // 2 ** J) ** 2
    spill = 2 * 8 * L * sum((Mp // 2 ** j1) ** 2 for j1 in range(J - 1))
    return 4 * side * side + out + spill


def group_fft_flops(level, ntasks, rows, cols, s_out):
    """5 n log2 n FLOPs per image of one launch group of the reference
    algorithm: the input stage does the FFT2 of the padded image and the
    small IFFT2 of S0; every path of an order-1 or order-2 group does the
    IFFT2 and the FFT2 at its resolution and the small IFFT2 of its output."""
    f2 = lambda m, n: 5.0 * m * n * math.log2(m * n)
    if level == 0:
        return f2(rows, cols) + f2(s_out, s_out)
    return ntasks * (2 * f2(rows, cols) + f2(s_out, s_out))


def s1d_algorithmic(mod):
    """(bytes, FLOPs) per signal of the 1-D local-averaging cascade
    (kymatio/scattering1d/core/scattering1d.py:40-107): input, output and one
    write + read of every first-order spectrum that has children; 5 n log2 n
    per FFT of the reference algorithm."""
    f = lambda n: 5.0 * n * math.log2(n) if n > 1 else 0.0
    n_pad, l2s = mod._N_padded, mod.log2_stride
    n_out = n_pad >> l2s
    j1s = [p['j'] for p in mod.psi1_f]
    j2s = [p['j'] for p in mod.psi2_f] if mod.max_order >= 2 else []
    flops = f(n_pad) + f(n_out)
    spill = 0
    for a in j1s:
        k1 = min(a, l2s)
        n1 = n_pad >> k1
        flops += 2 * f(n1) + f(n_out)
        kids = [b for b in j2s if b > a]
        if kids:
            spill += 2 * 8 * n1
        for b in kids:
            k2 = max(min(b, l2s) - k1, 0)
            flops += 2 * f(n1 >> k2) + f(n_out)
    C = len(mod._paths())
    return 4 * mod.shape[0] + 4 * C * n_out + spill, flops


def fp32_peak_tflops(dev, mhz):
    """FP32 pipe peak derived from the device: SMs x 128 FP32 lanes x 2 (FMA)
    x SM clock (the median sampled under load)."""
    import torch
    return torch.cuda.get_device_properties(dev).multi_processor_count * 128 * 2 * mhz * 1e6 / 1e12


def fft_flops_per_image(J=J, L=L, side=SIDE):
    """5 n log2 n convention over every 2-D FFT of the cascade."""
    Mp = ((side + 2 ** J) // 2 ** J + 1) * 2 ** J
    f = lambda m: 5.0 * m * m * math.log2(m * m)
    s = Mp // 2 ** J
    tot = f(Mp) + f(s)
    for j1 in range(J):
        m1 = Mp >> j1
        tot += L * (2 * f(m1) + f(s))
        for j2 in range(j1 + 1, J):
            m2 = Mp >> j2
            tot += L * L * (2 * f(m2) + f(s))
    return tot


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
         'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
         'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, index):
        self.index, self.proc, self.path = index, None, None

    def start(self):
        try:
            self.path = os.path.join(tempfile.gettempdir(), 'kym_bench_clocks_%d.csv' % os.getpid())
            self.f = open(self.path, 'w')
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.index), '--query-gpu=' + self.Q,
                                          '--format=csv,noheader,nounits', '-lms', '200'],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        for line in open(self.path):
            p = [t.strip() for t in line.split(',')]
            if len(p) >= 9:
                rows.append(p)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace('.', '').isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace('.', '').isdigit()]
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith('active')})
        load = [v for v in sm if mx and v > 0.5 * max(mx)] or sm
        return {'sm_mhz': statistics.median(load) if load else None, 'sm_max_mhz': max(mx) if mx else None,
                'reasons': reasons, 'samples': len(rows)}


_REF = {}


def reference_kymatio():
    """The reference package as pip-installed into baseline/_ref (its stock
    frontends, backends and filter banks), or None when it is not there."""
    if 'mod' in _REF:
        return _REF['mod']
    path = os.path.join(ROOT, 'baseline', '_ref')
    mod = None
    if os.path.isfile(os.path.join(path, 'kymatio', '__init__.py')):
        dont = sys.dont_write_bytecode
        sys.dont_write_bytecode = True
        sys.path.insert(0, path)
        try:
            import kymatio
            # the frontend modules directly: kymatio.torch also imports the
            # 3-D filter bank, whose scipy import fails on current scipy
            from kymatio.scattering1d.frontend import torch_frontend as _f1  # noqa: F401
            from kymatio.scattering2d.frontend import numpy_frontend as _n2  # noqa: F401
            from kymatio.scattering2d.frontend import torch_frontend as _f2  # noqa: F401
            mod = kymatio
        except Exception:
            mod = None
        finally:
            sys.path.remove(path)
            sys.dont_write_bytecode = dont
    _REF['mod'] = mod
    return mod


def _best_s(fn, repeats, warm=True):
    if warm:
        fn()
    best = float('inf')
    for _ in range(repeats):
        t = time.perf_counter()
        fn()
        best = min(best, time.perf_counter() - t)
    return best


def ref_torch_module(J_, shape, **kw):
    """The reference's stock torch frontend (CPU), built once per geometry."""
    key = ('t2d', J_, tuple(shape) if not isinstance(shape, int) else shape, tuple(sorted(kw.items())))
    if key not in _REF:
        kym = reference_kymatio()
        if isinstance(shape, int):
            from kymatio.scattering1d.frontend.torch_frontend import ScatteringTorch1D
            _REF[key] = ScatteringTorch1D(J_, shape, **kw)
        else:
            from kymatio.scattering2d.frontend.torch_frontend import ScatteringTorch2D
            _REF[key] = ScatteringTorch2D(J_, shape, **kw)
        assert kym is not None
    return _REF[key]


def cpu_reference_rate(n_img, threads, repeats=1, x=None):
    """Images/s of the reference's CPU implementation on n_img images of the
    workload (best of ``repeats`` after one warm-up): kymatio's stock
    ScatteringTorch2D in float32 on ``threads`` host threads when the
    reference is installed (kind "reference"), else the oracle port of its
    numpy backend in float32 (kind "port").  Returns (img/s, seconds, kind)."""
    import torch
    if x is None:
        x = grf_batch(n_img, seed=2)
    if reference_kymatio() is not None:
        torch.set_num_threads(threads)
        S = ref_torch_module(J, (SIDE, SIDE), L=L)
        xt = torch.from_numpy(x[:n_img])
        with torch.no_grad():
            best = _best_s(lambda: S(xt), repeats)
        return n_img / best, best, 'reference'
    import scipy.fft
    from oracle.scattering2d import Scattering2D as Oracle
    S = Oracle(J, (SIDE, SIDE), L=L)
    with scipy.fft.set_workers(threads):
        best = _best_s(lambda: S(x[:n_img]), repeats)
    return n_img / best, best, 'port'


def fp64_reference(x):
    """The FP64 reference output for images x: the reference's numpy frontend
    fed float64 input (its filters as it builds them), else the oracle port."""
    kym = reference_kymatio()
    if kym is not None:
        from kymatio.scattering2d.frontend.numpy_frontend import ScatteringNumPy2D
        return ScatteringNumPy2D(J, (x.shape[-2], x.shape[-1]), L=L)(x.astype(np.float64))
    from oracle.scattering2d import Scattering2D as Oracle
    return Oracle(J, (x.shape[-2], x.shape[-1]), L=L)(x.astype(np.float64))


def dist_init():
    import torch
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    if world > 1:
        import torch.distributed as dist
        backend = 'nccl' if torch.cuda.is_available() else 'gloo'
        dist.init_process_group(backend=backend)
    return world, rank, local


def max_over_ranks(v, world):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device='cuda' if torch.cuda.is_available() else 'cpu')
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def run_reference(args, world, rank):
    """The reference's own CPU implementation on the host cores: one step is
    one forward of kymatio's stock ScatteringTorch2D over the full batch."""
    if rank != 0:
        return
    import torch
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    x = grf_batch(BATCH, seed=2)
    kind = 'reference' if reference_kymatio() is not None else 'port'
    if kind == 'reference':
        S = ref_torch_module(J, (SIDE, SIDE), L=L)
        xt = torch.from_numpy(x)

        def step():
            with torch.no_grad():
                S(xt)
        what = ("kymatio's stock ScatteringTorch2D (torch %s on the CPU, fp32, %d threads), the full %d-image "
                'batch per step' % (torch.__version__, threads, BATCH))
    else:
        import scipy.fft
        from oracle.scattering2d import Scattering2D as Oracle
        So = Oracle(J, (SIDE, SIDE), L=L)

        def step():
            with scipy.fft.set_workers(threads):
                So(x)
        what = ('reference not installed in baseline/_ref: oracle port of its numpy backend, fp32, '
                'scipy.fft workers=%d, the full %d-image batch per step' % (threads, BATCH))
    for _ in range(args.warmup):
        step()
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        step()
        times.append(time.perf_counter() - t)
    value = BATCH * len(times) / sum(times)
    line = {'metric': METRIC, 'value': value, 'unit': 'img/s', 'n_gpus': args.gpus, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': 1e3 * sum(times) / len(times), 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic',
            'impl': 'reference',
            'config': {'workload': 'Scattering2D J=3 L=8 max_order=2, 256x256 GRF float32',
                       'global_batch': BATCH, 'per_gpu_batch': BATCH, 'parallelism': 'host cores'},
            'cpu_baseline': {'value': value, 'unit': 'img/s', 'cores': threads, 'kind': kind, 'sample': what},
            'e2e': {'value': value, 'unit': 'img/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)


def order_rel_l2(out, ref):
    """Relative L2 error per scattering order (S0, S1, S2 channel ranges)."""
    n1 = J * L
    res = []
    for sl in (slice(0, 1), slice(1, 1 + n1), slice(1 + n1, None)):
        a, b = out[:, sl].astype(np.float64), ref[:, sl]
        res.append(float(np.linalg.norm(a - b) / np.linalg.norm(b)))
    return res


def _time_ms(fn, steps, warmup, flush):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    tot = 0.0
    for _ in range(steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        tot += e0.elapsed_time(e1)
    return tot / steps


CTX = {'hbm_gbs': 6800.0, 'fp32_tflops': None, 'peak_source': 'fallback', 'cpu': True}


def _roofline(bytes_unit, flops_unit, rate, unit):
    """Both roofline terms of a whole workload at ``rate`` units/s."""
    r = {'bytes_per_%s' % unit: bytes_unit, 'gflop_per_%s_5nlogn' % unit: flops_unit / 1e9,
         'hbm': {'achieved_gbs': bytes_unit * rate / 1e9, 'peak_gbs': CTX['hbm_gbs'],
                 'frac': bytes_unit * rate / 1e9 / CTX['hbm_gbs'], 'peak_source': CTX['peak_source']}}
    if CTX['fp32_tflops']:
        r['fp32'] = {'achieved_tflops': flops_unit * rate / 1e12, 'peak_tflops': CTX['fp32_tflops'],
                     'frac': flops_unit * rate / 1e12 / CTX['fp32_tflops'],
                     'peak_source': 'derived: SMs x 128 lanes x 2 x median SM clock'}
    return r


def _ref_cpu(fn_build, fn_run, n, unit, repeats=2):
    """The reference's stock torch frontend on the host cores (all threads,
    no_grad, best of ``repeats`` after one warm-up): units/s, or None."""
    if not CTX['cpu'] or reference_kymatio() is None:
        return None
    import torch
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    mod = fn_build()
    with torch.no_grad():
        sec = _best_s(lambda: fn_run(mod), repeats)
    return {'value': n / sec, 'unit': unit, 'cores': threads, 'kind': 'reference',
            'sample': '%d per call, torch %s CPU fp32, best of %d' % (n, torch.__version__, repeats)}


def _extra_s2d_32(dev, flush, steps, warmup):
    """32x32, J=2, batch 128, U[0,1) seed 0 (plain and tensor-core forms)."""
    import torch
    from kymatio_gb300 import Scattering2D
    xn = np.random.default_rng(0).random((128, 32, 32)).astype(np.float32)
    x = torch.from_numpy(xn).to(dev)
    S = Scattering2D(2, (32, 32)).to(dev)
    ms = _time_ms(lambda: S(x), steps, warmup, flush)
    S.tensor_cores = True
    ms_tc = _time_ms(lambda: S(x), steps, warmup, flush)
    rate = 128 / ms * 1e3
    return {'img_s': rate, 'img_s_tc': 128 / ms_tc * 1e3,
            'roofline_plain': _roofline(algorithmic_bytes_per_image(2, 8, 32), fft_flops_per_image(2, 8, 32),
                                        rate, 'img'),
            'cpu_baseline': _ref_cpu(lambda: ref_torch_module(2, (32, 32)),
                                     lambda m: m(torch.from_numpy(xn)), 128, 'img/s', repeats=3)}


def _extra_s1d_8192(dev, flush, steps, warmup):
    """1-D N=8192, J=6, Q=(8,1), T=64, batch 256: white noise plus a linear chirp, seed 1."""
    import torch
    from kymatio_gb300.scattering1d import Scattering1D
    rng = np.random.default_rng(1)
    N, B = 8192, 256
    t = np.arange(N)
    f0 = rng.uniform(0.01, 0.1, B)[:, None]
    f1 = rng.uniform(0.1, 0.4, B)[:, None]
    sig = rng.standard_normal((B, N)) + np.cos(2 * np.pi * (f0 * t + (f1 - f0) * t ** 2 / (2 * N)))
    xn = sig.astype(np.float32)
    xs = torch.from_numpy(xn).to(dev)
    S1 = Scattering1D(6, N, Q=(8, 1), T=64).to(dev)
    ms = _time_ms(lambda: S1(xs), steps, warmup, flush)
    rate = B / ms * 1e3
    b, f = s1d_algorithmic(S1)
    return {'sig_s': rate, 'roofline': _roofline(b, f, rate, 'signal'),
            'cpu_baseline': _ref_cpu(lambda: ref_torch_module(6, N, Q=(8, 1), T=64),
                                     lambda m: m(torch.from_numpy(xn)), B, 'signals/s')}


def _extra_fwd_bwd_128(dev, flush, steps, warmup):
    """128x128, J=4, batch 32 (U[0,1) seed 3, upstream N(0,1)): forward vs
    forward + hand-written backward, saved and recompute policies."""
    import torch
    from kymatio_gb300 import Scattering2D
    rng = np.random.default_rng(3)
    x4 = torch.from_numpy(rng.random((32, 128, 128)).astype(np.float32)).to(dev)
    g4 = torch.from_numpy(rng.standard_normal((32, 417, 8, 8)).astype(np.float32)).to(dev)
    S4 = Scattering2D(4, (128, 128)).to(dev)
    fwd = _time_ms(lambda: S4(x4), steps, warmup, flush)
    xr = x4.clone().requires_grad_()

    def fb():
        xr.grad = None
        S4(xr).backward(g4)
    fwdbwd = _time_ms(fb, steps, warmup, flush)
    S4.activation_budget = 0  # recompute form: only x kept, spectra and y recomputed
    fwdbwd_rc = _time_ms(fb, steps, warmup, flush)
    cpu = None
    if CTX['cpu'] and reference_kymatio() is not None:
        threads = os.cpu_count() or 1
        torch.set_num_threads(threads)
        R = ref_torch_module(4, (128, 128))
        xc, gc = x4.cpu(), g4.cpu()
        with torch.no_grad():
            f_s = _best_s(lambda: R(xc), 2)
        xq = xc.clone().requires_grad_()

        def rfb():
            xq.grad = None
            R(xq).backward(gc)
        fb_s = _best_s(rfb, 2)
        cpu = {'fwd_ms': f_s * 1e3, 'fwd_bwd_ms': fb_s * 1e3, 'ratio': fb_s / f_s, 'cores': threads,
               'kind': 'reference', 'sample': 'the full batch of 32, torch %s CPU autograd, fp32' % torch.__version__}
    return {'fwd_ms': fwd, 'fwd_bwd_ms': fwdbwd, 'ratio': fwdbwd / fwd,
            'policy': 'saved modulus inputs, %.1f MB (4 GiB budget)' % (S4._saved_bytes(32) / 1e6),
            'fwd_bwd_ms_recompute': fwdbwd_rc, 'ratio_recompute': fwdbwd_rc / fwd, 'cpu_baseline': cpu}


#: input slices of the end-to-end host forward
E2E_PARTS = 1


def _lib_handle():
    from kymatio_gb300 import _lib
    return _lib.load()


def _extra_mixed_512(dev, flush, steps, warmup):
    """512 images, sides drawn from {32,64,128,256}, seed 4: per-size launches
    vs one CUDA graph over grouped streams (plain and tensor-core forms)."""
    import torch
    from kymatio_gb300 import Scattering2D
    from kymatio_gb300.batching import MixedScattering2D, default_J
    rng = np.random.default_rng(4)
    sides = rng.choice([32, 64, 128, 256], size=512)
    imgs = [torch.from_numpy(rng.random((s, s)).astype(np.float32)).to(dev) for s in sides]
    groups = {}
    for im in imgs:
        groups.setdefault(int(im.shape[-1]), []).append(im)
    xs = {s: torch.stack(v) for s, v in groups.items()}
    mods = {s: Scattering2D(default_J(s), (s, s)).to(dev) for s in xs}
    seq = _time_ms(lambda: [mods[s](xs[s]) for s in sorted(xs)], steps, warmup, flush)
    mix = MixedScattering2D(list(xs)).to(dev)
    gr = _time_ms(lambda: mix.forward_grouped(xs), steps, warmup, flush)
    mixt = MixedScattering2D(list(xs), tensor_cores=True).to(dev)
    grt = _time_ms(lambda: mixt.forward_grouped(xs), steps, warmup, flush)
    # autotuned: chunk and, in the tensor-core form, the kernel form per size
    # (tuning cache in a temporary directory, so the run starts cold)
    import tempfile
    old_cache = os.environ.get('KYMATIO_GB300_CACHE')
    with tempfile.TemporaryDirectory() as tmp:
        os.environ['KYMATIO_GB300_CACHE'] = tmp
        mixa = MixedScattering2D(list(xs), tensor_cores=True, tune=True).to(dev)
        mixa.forward_grouped(xs)
        lib = _lib_handle()
        tuned = {int(k): sum(lib.kym_s2d_group_uses_tc(m._get_plan().h, g) > 0
                             for g in range(lib.kym_s2d_group_count(m._get_plan().h)))
                 for k, m in mixa.mods.items()}
        gra = _time_ms(lambda: mixa.forward_grouped(xs), steps, warmup, flush)
    if old_cache is None:
        os.environ.pop('KYMATIO_GB300_CACHE', None)
    else:
        os.environ['KYMATIO_GB300_CACHE'] = old_cache
    cpu = None
    if CTX['cpu'] and reference_kymatio() is not None:
        # one reference module per side (its frontend fixes the shape), on a
        # sample of 4 images per side, weighted by the batch's counts
        threads = os.cpu_count() or 1
        torch.set_num_threads(threads)
        tot = 0.0
        for s_, v in sorted(groups.items()):
            R = ref_torch_module(default_J(s_), (s_, s_))
            xc = xs[s_][:4].cpu()
            with torch.no_grad():
                tot += _best_s(lambda: R(xc), 1) / xc.shape[0] * len(v)
        cpu = {'value': 512 / tot, 'unit': 'img/s', 'cores': threads, 'kind': 'reference',
               'sample': '4 images per side, one stock ScatteringTorch2D per side, time scaled to the counts'}
    return {'img_s_per_size_sequential': 512 / seq * 1e3, 'img_s_graph': 512 / gr * 1e3,
            'img_s_graph_tc': 512 / grt * 1e3, 'img_s_graph_tc_autotuned': 512 / gra * 1e3,
            'autotuned_tensor_core_groups': {str(k): v for k, v in sorted(tuned.items())},
            'counts': {str(s): len(v) for s, v in sorted(groups.items())}, 'cpu_baseline': cpu}


def _extra_jtfs_8192(dev, flush, steps, warmup):
    """Joint time-frequency scattering, N=8192, J=6, J_fr=2, Q=(8,2), batch 64,
    'time' format (the chirp signals of the 1-D workload), op by op over the
    CUDA op surface."""
    import torch
    from kymatio_gb300.jtfs import TimeFrequencyScattering
    rng = np.random.default_rng(1)
    N, B = 8192, 64
    t = np.arange(N)
    f0 = rng.uniform(0.01, 0.1, B)[:, None]
    f1 = rng.uniform(0.1, 0.4, B)[:, None]
    sig = (rng.standard_normal((B, N)) + np.cos(2 * np.pi * (f0 * t + (f1 - f0) * t ** 2 / (2 * N)))).astype(np.float32)
    xs = torch.from_numpy(sig).to(dev)
    S = TimeFrequencyScattering(J=6, J_fr=2, Q=(8, 2), shape=N).to(dev)
    with torch.no_grad():
        ms = _time_ms(lambda: S(xs), steps, warmup, flush)
        S.graph = True  # the same forward replayed from one CUDA graph
        ms_graph = _time_ms(lambda: S(xs), steps, warmup, flush)
        S.graph = False
    cpu = None
    if CTX['cpu'] and reference_kymatio() is not None:
        from kymatio.scattering1d.frontend.torch_frontend import TimeFrequencyScatteringTorch
        threads = os.cpu_count() or 1
        torch.set_num_threads(threads)
        R = TimeFrequencyScatteringTorch(J=6, J_fr=2, Q=(8, 2), shape=N)
        xc = torch.from_numpy(sig[:8])
        with torch.no_grad():
            sec = _best_s(lambda: R(xc), 1)
        cpu = {'value': 8 / sec, 'unit': 'signals/s', 'cores': threads, 'kind': 'reference',
               'sample': '8 signals, stock TimeFrequencyScatteringTorch, torch %s CPU fp32' % torch.__version__}
    return {'sig_s': B / ms * 1e3, 'sig_s_graph': B / ms_graph * 1e3, 'channels': int(S(xs[:1]).shape[-2]),
            'cpu_baseline': cpu}


def _extra_filter_bank(dev, flush, steps, warmup):
    """Construction of the 2-D filter bank at 256x256 J=3 (padded 272, L=8)
    and 256x256 J=4 (padded 288): the host build (bit for bit the
    reference's), the device build (FP64 on the GPU), and the reference's
    own constructor on the host cores."""
    import torch
    from kymatio_gb300.filter_bank import filter_bank_2d, filter_bank_2d_device
    res = {}
    for (Mp, J_) in ((272, 3), (288, 4)):
        filter_bank_2d.cache_clear()
        t = time.perf_counter()
        filter_bank_2d(Mp, Mp, J_, 8)
        host_s = time.perf_counter() - t
        filter_bank_2d_device(Mp, Mp, J_, 8)  # first call: module load
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(3):
            filter_bank_2d_device(Mp, Mp, J_, 8)
        torch.cuda.synchronize()
        dev_s = (time.perf_counter() - t) / 3
        r = {'host_s': host_s, 'device_s': dev_s}
        if CTX['cpu'] and reference_kymatio() is not None:
            from kymatio.scattering2d.filter_bank import filter_bank as ref_bank
            t = time.perf_counter()
            ref_bank(Mp, Mp, J_, 8)
            r['reference_host_s'] = time.perf_counter() - t
        res['padded_%d_J%d' % (Mp, J_)] = r
    return res


EXTRAS = {
    'filter_bank_construction': _extra_filter_bank,
    'scattering2d_32x32_J2_b128': _extra_s2d_32,
    'jtfs_8192_J6_Jfr2_Q8_2_b64': _extra_jtfs_8192,
    'scattering1d_8192_J6_Q8_T64_b256': _extra_s1d_8192,
    'scattering2d_128x128_J4_b32_fwd_bwd': _extra_fwd_bwd_128,
    'mixed_512_sides_32_64_128_256': _extra_mixed_512,
}


def extras(dev, flush, steps=5, warmup=3, names=None):
    """The other workloads (all of EXTRAS, or the named ones)."""
    return {n: f(dev, flush, steps, warmup) for n, f in EXTRAS.items() if names is None or n in names}


def run_ours(args, world, rank, local):
    import ctypes
    import torch
    from kymatio_gb300 import Scattering2D, _lib
    torch.cuda.set_device(local)
    dev = torch.device('cuda', local)
    lib = _lib.load()
    x_np = grf_batch(BATCH, seed=2 + rank)
    x_host = torch.from_numpy(x_np).pin_memory()
    x = x_host.to(dev)
    S = Scattering2D(J, (SIDE, SIDE), L=L).to(dev)
    if args.chunk:
        S.set_chunk(args.chunk)
    plan = S._get_plan()
    ngroups = lib.kym_s2d_group_count(plan.h)
    ginfo = []
    for g in range(ngroups):
        v = [ctypes.c_int() for _ in range(6)]
        lib.kym_s2d_group_info(plan.h, g, *[ctypes.byref(i) for i in v])
        ginfo.append([i.value for i in v] + [lib.kym_s2d_group_uses_tc(plan.h, g),
                                             lib.kym_s2d_group_kernels(plan.h, g, 1)])
    chunk = lib.kym_s2d_get_chunk(plan.h)
    n_chunks = -(-BATCH // min(chunk, BATCH))
    # kernels of the tensor-core form per step, as the library launches them
    # (chunks, line-split and shared-fold sub-launches)
    launches = [lib.kym_s2d_group_launches(plan.h, g, BATCH, 1) for g in range(ngroups)]
    launches_per_step = sum(launches)
    out = torch.empty((BATCH, S._channels) + S._out_hw, device=dev)
    ws_bytes = lib.kym_s2d_workspace_bytes(plan.h, BATCH)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
    ptrs = S._filter_ptrs()
    lr, lc = S._lowpass_ptrs()
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)  # > L2 (129 MB)
    stream = torch.cuda.current_stream(dev)
    gms = (ctypes.c_float * ngroups)()

    def step(form, timed_groups):
        g = gms if timed_groups else None
        ng = ngroups if timed_groups else 0
        if form == 'tc':
            _lib.check(lib.kym_s2d_forward_tc(plan.h, x.data_ptr(), out.data_ptr(), BATCH, ptrs, S._n_filters, lr, lc,
                                              J, ws.data_ptr(), ws_bytes, S._tc_status.data_ptr(),
                                              stream.cuda_stream, g, ng), 'forward_tc')
        elif timed_groups:
            _lib.check(lib.kym_s2d_forward_timed(plan.h, x.data_ptr(), out.data_ptr(), BATCH, ptrs, S._n_filters,
                                                 ws.data_ptr(), ws_bytes, stream.cuda_stream, gms, ngroups),
                       'forward_timed')
        else:
            _lib.check(lib.kym_s2d_forward(plan.h, x.data_ptr(), out.data_ptr(), BATCH, ptrs, S._n_filters,
                                           ws.data_ptr(), ws_bytes, stream.cuda_stream), 'forward')

    def measure(form):
        for _ in range(args.warmup):
            step(form, False)
        torch.cuda.synchronize()
        barrier(world)
        times = []
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step(form, False)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        barrier(world)
        gtot = np.zeros(ngroups)
        for _ in range(args.steps):
            flush.zero_()
            step(form, True)
            gtot += np.array([gms[i] for i in range(ngroups)])
        return max_over_ranks(sum(times) / len(times), world), gtot / args.steps

    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, 'MEASURED_PEAKS.json')))
    except Exception:
        pass
    CTX['hbm_gbs'] = peaks.get('hbm_gbs', 6800.0)
    CTX['peak_source'] = 'measured' if 'hbm_gbs' in peaks else 'fallback'
    CTX['cpu'] = not args.no_cpu
    # precision of each form on two images vs the FP64 reference (the
    # reference's numpy frontend fed float64)
    prec = {}
    if rank == 0 and not args.no_cpu:
        # the first and the last image: the last one sits in the last chunk and
        # the last sub-launch of the line-split groups
        pick = [0, BATCH - 1] if BATCH > 1 else [0]
        ref = fp64_reference(x_np[pick])
        for form in ('plain', 'tc', 'tc_dft'):
            prev = lib.kym_set_tc_dft(1 if form == 'tc_dft' else 0)
            step('plain' if form == 'plain' else 'tc', False)
            torch.cuda.synchronize()
            lib.kym_set_tc_dft(prev)
            prec[form] = order_rel_l2(out[pick].cpu().numpy(), ref)
    sampler = ClockSampler(local)
    sampler.start()
    t_plain, g_plain = measure('plain')
    t_tc, g_tc = measure('tc')
    # the DFT-GEMM form of the 68x68 groups (opt-in), measured beside the default form
    prev_dft = lib.kym_set_tc_dft(1)
    t_dft, g_dft = measure('tc')
    lib.kym_set_tc_dft(prev_dft)
    clocks = sampler.stop()
    tc_status = S.tensor_core_status()
    value = BATCH * world / (t_tc / 1e3)
    value_plain = BATCH * world / (t_plain / 1e3)
    # ---- end to end through the public API (tensor-core form): pinned host in, host out
    S.tensor_cores = True
    out_host = torch.empty((BATCH, S._channels) + S._out_hw, dtype=torch.float32).pin_memory()

    def e2e_step(kind):
        if kind == 'host':  # Scattering2D.forward_host: transfers overlapped with the cascade
            S.forward_host(x_host, out_host, parts=args.e2e_parts, sync=False)
        else:  # tensor API: copy in, forward, copy out, one after the other
            out_host.copy_(S(x_host.to(dev, non_blocking=True)), non_blocking=True)

    fe0, fe1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    fe0.record(stream)
    for _ in range(args.steps):
        flush.zero_()
    fe1.record(stream)
    torch.cuda.synchronize()
    flush_ms = fe0.elapsed_time(fe1)
    e2e_ms = {}
    for kind in ('tensor', 'host'):
        for _ in range(max(1, args.warmup)):
            e2e_step(kind)
        torch.cuda.synchronize()
        barrier(world)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            flush.zero_()
            e2e_step(kind)
        e1.record(stream)
        torch.cuda.synchronize()
        e2e_ms[kind] = max_over_ranks((e0.elapsed_time(e1) - flush_ms) / args.steps, world)
    e2e = BATCH * world / (e2e_ms['host'] / 1e3)
    e2e_tensor = BATCH * world / (e2e_ms['tensor'] / 1e3)
    # ---- roofline of the dominant launch group of the tensor-core form -----------
    # (one launch = all the kernels of the group over one chunk of images)
    per_launch = [g_tc[g] / (1 if gi[0] == 0 else n_chunks) for g, gi in enumerate(ginfo)]
    dom = int(np.argmax(g_tc))
    lvl, ntasks, rows, cols, fold, cl, uses_tc, nkern = ginfo[dom]
    imgs_per_launch = BATCH if lvl == 0 else min(chunk, BATCH)
    side_out = SIDE // 2 ** J
    Mp = ((SIDE + 2 ** J) // 2 ** J + 1) * 2 ** J
    # algorithmic bytes of one launch: every source spectrum once per image (an
    # order-1 group reads the input spectrum, an order-2 group its ntasks / L
    # parents) -- the non-redundant half of it, rows 0 .. P/2, a real image's
    # spectrum being Hermitian (the fold reads that much) --, the output
    # channels, the parent spectra an order-1 group writes, and each distinct
    # filter once per launch (L wavelets, one low-pass)
    if lvl == 0:
        bytes_launch = imgs_per_launch * (4 * SIDE * SIDE + 8 * rows * cols + 4 * side_out ** 2)
    else:
        src = fold * fold * rows * cols
        src_half = (fold * rows // 2 + 1) * fold * cols
        n_src = 1 if lvl == 1 else max(1, ntasks // L)
        spill_w = ntasks * 8 * rows * cols if (lvl == 1 and not uses_tc and J > 1 and rows > (Mp >> (J - 1))) else 0
        bytes_launch = imgs_per_launch * (n_src * 8 * src_half + ntasks * 4 * side_out ** 2 + spill_w) + \
            min(ntasks, L) * 4 * src + 4 * rows * cols
    dur_s = per_launch[dom] / 1e3
    hbm_peak = CTX['hbm_gbs']
    achieved = bytes_launch / dur_s / 1e9
    s_out = Mp // 2 ** J
    flops_launch = imgs_per_launch * group_fft_flops(lvl, ntasks, rows, cols, s_out)
    sm_mhz = (clocks or {}).get('sm_mhz') or peaks.get('sm_max_mhz', 2070.0)
    CTX['fp32_tflops'] = fp32_peak_tflops(dev, sm_mhz)
    # DRAM bytes of one launch of this group, from the committed ncu summary
    # (null when the dominant group has no capture)
    traffic = None
    form_key = 'tc' if uses_tc else ('lines' if nkern > 1 else 'fused')
    tkey = 'L%d_%dx%d_f%d_%s' % (lvl, rows, cols, fold, form_key)
    tf = os.path.join(ROOT, 'profiles', 'dominant_traffic.json')
    if os.path.exists(tf):
        try:
            traffic = json.load(open(tf)).get('kernels', {}).get(tkey, {}).get('bytes_per_launch')
        except Exception:
            traffic = None
    flops_img = fft_flops_per_image()
    # each form within its bar against the FP64 reference (relative L2 per order)
    bars = {'plain': 1e-5, 'tc': 5e-5, 'tc_dft': 5e-5}
    prec_ok = None if not prec else all(max(v) <= bars[k] for k, v in prec.items())
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        rate, sec, kind = cpu_reference_rate(BATCH, threads, repeats=1, x=x_np)
        cpu = {'value': rate, 'unit': 'img/s', 'cores': threads, 'kind': kind,
               'sample': ('the full %d-image batch (%.1f s after one warm-up), ' % (BATCH, sec)) +
                         ("kymatio's stock ScatteringTorch2D, torch CPU fp32, %d threads" % threads
                          if kind == 'reference' else
                          'oracle port of the reference numpy backend in fp32, scipy.fft workers=%d' % threads)}
    extra = None
    if rank == 0 and world == 1 and not args.no_extras:
        extra = extras(dev, flush)
    if rank == 0:
        line = {
            'metric': METRIC, 'value': value, 'unit': 'img/s', 'n_gpus': world, 'steps': args.steps,
            'warmup': args.warmup, 'ms_per_step': t_tc, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic',
            'config': {'workload': 'Scattering2D J=3 L=8 max_order=2, 256x256 GRF float32, tensor-core '
                                   'split-precision form (tcgen05 bf16 hi/lo, fp32 accumulate)',
                       'global_batch': BATCH * world, 'per_gpu_batch': BATCH, 'chunk': chunk,
                       'l2': 'flushed (256 MB write) between timed steps', 'parallelism': 'replicas x%d' % world},
            'plain_fp32': {'value': value_plain, 'unit': 'img/s', 'ms_per_step': t_plain,
                           'rel_l2_vs_fp64': prec.get('plain'),
                           'group_ms_per_step': [round(v, 4) for v in g_plain]},
            'tc_vs_plain': value / value_plain,
            'tc_dft_gemm': {'value': BATCH * world / (t_dft / 1e3), 'unit': 'img/s', 'ms_per_step': t_dft,
                            'rel_l2_vs_fp64': prec.get('tc_dft'),
                            'group_ms_per_step': [round(v, 4) for v in g_dft],
                            'groups': 'the 68x68 groups (order 1 j1=2, order 2 (0,2) and (1,2)) as DFT-GEMMs '
                                      'on tcgen05 after a shared-source fold pass; other groups as in the '
                                      'tensor-core form'},
            'rel_l2_vs_fp64': prec.get('tc'), 'rel_l2_orders': ['S0', 'S1', 'S2'],
            'tc_status': tc_status,
            'e2e': {'value': e2e, 'unit': 'img/s', 'h2d_bytes_per_step': int(x_host.numel() * 4),
                    'd2h_bytes_per_step': int(out_host.numel() * 4),
                    'api': 'Scattering2D.forward_host (kym_s2d_forward_host), pinned host buffers, input in '
                           '%d slices, each group\'s channels copied back as it finishes' % args.e2e_parts,
                    'tensor_api': {'value': e2e_tensor, 'unit': 'img/s',
                                   'api': 'x_host.to(cuda) -> Scattering2D -> copy to pinned host, in sequence'}},
            'gpu_launches': launches_per_step * args.steps,
            'roofline': {'bound': 'hbm', 'achieved': achieved, 'peak': hbm_peak, 'unit': 'GB/s',
                         'frac': achieved / hbm_peak, 'traffic': traffic,
                         'fp32': {'achieved_tflops': flops_launch / dur_s / 1e12,
                                  'peak_tflops': CTX['fp32_tflops'],
                                  'frac': flops_launch / dur_s / 1e12 / CTX['fp32_tflops'],
                                  'flops': '5 n log2 n per FFT of the reference algorithm',
                                  'peak_source': 'derived: SMs x 128 lanes x 2 x median SM clock %.0f MHz'
                                                 % sm_mhz},
                         'step': _roofline(algorithmic_bytes_per_image(), flops_img, value / world, 'img'),
                         'kernel': 'cascade group %d (level %d, %dx%d, fold %d, %d tasks%s)'
                                   % (dom, lvl, rows, cols, fold, ntasks,
                                      ', tensor-core' if uses_tc else
                                      (', %d line-split kernels' % nkern if nkern > 1 else ', one fused kernel')),
                         'kernel_ms_per_launch': per_launch[dom],
                         'peak_source': 'measured' if 'hbm_gbs' in peaks else 'fallback'},
            'fp32_fft': {'gflop_per_img_5nlogn': flops_img / 1e9,
                         'achieved_tflops_plain': flops_img * value_plain / world / 1e12},
            'precision_ok': prec_ok,
            'group_ms_per_step': [round(v, 4) for v in g_tc],
            'clocks': clocks,
            'cpu_baseline': cpu,
            'extras': extra,
        }
        print(json.dumps(line), flush=True)
        if prec_ok is False:
            sys.stderr.write('precision above its bar: %s\n' % json.dumps(prec))
            sys.exit(3)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=20)
    ap.add_argument('--warmup', type=int, default=5)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--chunk', type=int, default=0)
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--no-extras', action='store_true', help='skip the other workloads')
    ap.add_argument('--batch', type=int, default=64, help='images per GPU (64 is the benchmark workload)')
    ap.add_argument('--extra', choices=sorted(EXTRAS), default=None,
                    help='run only this other workload (for profiling) and print its JSON line')
    ap.add_argument('--forwards', default=None,
                    help='comma-separated forms (plain, tc): run --repeat forwards of each on the benchmark batch '
                         '(--batch images) and exit; for ncu launch lists and captures')
    ap.add_argument('--repeat', type=int, default=3)
    ap.add_argument('--e2e-parts', type=int, default=E2E_PARTS,
                    help='input slices of the end-to-end host forward')
    args = ap.parse_args()
    global BATCH
    BATCH = args.batch
    args.warmup = max(args.warmup, 3)
    if args.impl == 'reference':
        world, rank = int(os.environ.get('WORLD_SIZE', '1')), int(os.environ.get('RANK', '0'))
        run_reference(args, world, rank)
        return
    if args.forwards:
        import torch
        from kymatio_gb300 import Scattering2D
        dev = torch.device('cuda', 0)
        x = torch.from_numpy(grf_batch(BATCH, seed=2)).to(dev)
        for form in args.forwards.split(','):
            S = Scattering2D(J, (SIDE, SIDE), L=L, backend={'plain': 'torch', 'tc': 'torch_tc'}[form]).to(dev)
            for _ in range(args.repeat):
                S(x)
        torch.cuda.synchronize()
        return
    if args.extra:
        import torch
        dev = torch.device('cuda', 0)
        CTX['cpu'] = not args.no_cpu
        flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
        print(json.dumps({'extra': args.extra, **extras(dev, flush, args.steps, args.warmup, [args.extra])[args.extra]}))
        return
    world, rank, local = dist_init()
    run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == '__main__':
    main()
