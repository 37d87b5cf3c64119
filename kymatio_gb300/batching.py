"""Mixed-size batches: one CUDA-graph launch over images of several sizes.

``MixedScattering2D`` takes images of different sides N (with J chosen per
side, by default J = min(log2 N - 3, 4)), groups them by size, and runs every
group's fused cascade on its own CUDA stream.  The whole batch is captured
once into a single CUDA graph (fork/join over the streams); later batches
with the same composition replay it with one host launch, the size groups
running concurrently on the GPU.  An autotuner (``autotune``) picks each
size's parent-spectrum chunk (images per order-2 pass) and, when the
tensor-core form is asked for, which launch groups run their tensor-core
kernel and which the plain FP32 kernel (the more precise of the two, so either
meets the tensor-core form's bar), by timing candidates; the choices are
cached per (N, J, L, form, batch bucket) in a JSON file.
"""
import json
import math
import os
import threading

import torch

from .scattering2d import Scattering2D

_CACHE_LOCK = threading.Lock()


def cache_path():
    base = os.environ.get('KYMATIO_GB300_CACHE') or os.path.join(os.path.expanduser('~'), '.cache', 'kymatio_gb300')
    return os.path.join(base, 'autotune.json')


def _load_cache():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except Exception:
        return {}


def _store_cache(entries):
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + '.tmp'
        with open(tmp, 'w') as f:
            json.dump(entries, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass  # a read-only home leaves the in-process cache only


def autotune(module, batch, steps=3, candidates=None):
    """Time chunk sizes (images per order-2 pass) for ``module`` at ``batch``
    images and keep the fastest; for a module in the tensor-core form, then
    time every launch group in its tensor-core and its plain kernel and keep
    the faster per group (``module.set_group_tensor_cores``).  Cached per (N,
    J, L, form, batch bucket).  Returns the chosen chunk."""
    from . import _lib
    form = 'tc' if module.tensor_cores else 'plain'
    bucket = 1 << max(0, math.ceil(math.log2(max(1, batch))))
    key = '%dx%d/J%d/L%d/%s/f32/b%d' % (module.shape[0], module.shape[1], module.J, module.L, form, bucket)
    with _CACHE_LOCK:
        entries = _load_cache()
    if key in entries:
        module.set_chunk(entries[key]['chunk'])
        if 'tc_groups' in entries[key]:
            module.set_group_tensor_cores(entries[key]['tc_groups'])
        return entries[key]['chunk']
    dev = module.tensor0.device
    plan = module._get_plan()
    lib = _lib.load()
    default = lib.kym_s2d_get_chunk(plan.h)
    if candidates is None:
        candidates = sorted({max(1, c) for c in (default // 4, default // 2, default, default * 2, batch)})
    x = torch.rand((batch,) + module.shape, device=dev)
    best = None
    with torch.no_grad():
        for c in candidates:
            module.set_chunk(c)
            module(x)
            torch.cuda.synchronize(dev)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(steps):
                module(x)
            e1.record()
            e1.synchronize()
            ms = e0.elapsed_time(e1) / steps
            if best is None or ms < best[1]:
                best = (c, ms)
        module.set_chunk(best[0])
        entry = {'chunk': best[0], 'ms': best[1]}
        if module.tensor_cores:
            ng = lib.kym_s2d_group_count(plan.h)
            module.set_group_tensor_cores([True] * ng)
            module(x)
            t_on = module.group_times(x, steps)
            module.set_group_tensor_cores([False] * ng)
            module(x)
            t_off = module.group_times(x, steps)
            mask = [a <= b for a, b in zip(t_on, t_off)]
            module.set_group_tensor_cores(mask)
            entry['tc_groups'] = mask
    with _CACHE_LOCK:
        entries = _load_cache()
        entries[key] = entry
        _store_cache(entries)
    return best[0]


def default_J(N):
    return max(1, min(int(math.log2(N)) - 3, 4))


class MixedScattering2D(torch.nn.Module):
    """Scattering2D over a batch of square images of several sides.

    forward(images) takes a list of (N, N) float32 CUDA tensors (any order of
    sides) and returns the list of their (C_N, N/2^J, N/2^J) outputs, in the
    input order.  ``graph=True`` captures the grouped launches into one CUDA
    graph per batch composition; ``tensor_cores=True`` runs the split-precision
    form where a size has it.
    """

    def __init__(self, sides, L=8, max_order=2, J_of=default_J, tensor_cores=False, graph=True, tune=False):
        super().__init__()
        self.sides = sorted(set(int(s) for s in sides))
        self.mods = torch.nn.ModuleDict()
        for s in self.sides:
            m = Scattering2D(J_of(s), (s, s), L=L, max_order=max_order)
            m.tensor_cores = tensor_cores
            self.mods[str(s)] = m
        self.graph = graph
        self.tune = tune
        self._graphs = {}
        self._tuned = set()

    def _groups(self, images):
        idx = {}
        for i, im in enumerate(images):
            idx.setdefault(int(im.shape[-1]), []).append(i)
        return idx

    def _run_groups(self, xs, streams):
        outs = {}
        cur = torch.cuda.current_stream()
        for (s, x), st in zip(xs.items(), streams):
            st.wait_stream(cur)
            with torch.cuda.stream(st):
                outs[s] = self.mods[str(s)]._forward_raw(x)
        for st in streams:
            cur.wait_stream(st)
        return outs

    def forward_grouped(self, xs, copy=True):
        """xs: {side: (B_s, side, side) tensor} -> {side: output}, one graph launch.

        With ``copy=False`` the returned tensors are the graph's own output
        buffers: the next call with the same composition overwrites them.
        By default they are copied out first."""
        key = tuple(sorted((s, tuple(x.shape)) for s, x in xs.items()))
        dev = next(iter(xs.values())).device
        if self.tune and key not in self._tuned:  # once per composition
            for s, x in xs.items():
                autotune(self.mods[str(s)], x.shape[0])
            self._tuned.add(key)
        if not self.graph:
            streams = [torch.cuda.Stream(dev) for _ in xs]
            return self._run_groups(xs, streams)  # fresh outputs every call
        if key not in self._graphs:
            static_in = {s: x.clone() for s, x in xs.items()}
            streams = [torch.cuda.Stream(dev) for _ in xs]
            # warm-up outside capture: plans, device tables and kernel attributes
            self._run_groups(static_in, streams)
            torch.cuda.synchronize(dev)
            g = torch.cuda.CUDAGraph()
            cap = torch.cuda.Stream(dev)
            cap.wait_stream(torch.cuda.current_stream(dev))
            with torch.cuda.graph(g, stream=cap):
                static_out = self._run_groups(static_in, streams)
            self._graphs[key] = (g, static_in, static_out)
        g, static_in, static_out = self._graphs[key]
        for s, x in xs.items():
            static_in[s].copy_(x)
        g.replay()
        if not copy:
            return static_out
        return {s: o.clone() for s, o in static_out.items()}

    def forward(self, images):
        idx = self._groups(images)
        xs = {s: torch.stack([images[i] for i in ids]) for s, ids in idx.items()}
        outs = self.forward_grouped(xs)
        res = [None] * len(images)
        for s, ids in idx.items():
            for k, i in enumerate(ids):
                res[i] = outs[s][k]
        return res
