"""The MLP sun-transmittance surrogate: model handle, training-set generation
and training, all on the GPU through libcloudgb (features, exact-cone labels,
the fused FP16 tensor-core training step and Adam are the library's kernels).

Training data: scenes from the small workload's generator family (centres
uniform in a ball of radius 0.35, per-board density U[0.5, 1]) with the board
count and radius scale varied to span the small and the 1080p workloads,
voxelized at the evaluation resolution; sample positions are the view samples
the renderer's march pass records from random orbit views (kept with
probability proportional to their compositing weight T*alpha); labels are
the exact transmittance cone's optical depth at those positions.
"""
import ctypes
import math
import os

import numpy as np

from . import _lib, configs, scene
from ._lib import check, load

N_FEATURES = _lib.MLP_FEATURES
N_PARAMS = _lib.MLP_PARAMS


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


DEFAULT_LAYERS = _lib.MLP_DEFAULT_LAYERS


class SunMLP:
    """cg_mlp handle: 16 -> 64 [-> 64 [-> 64]] -> 1, SiLU, with 3 (default), 2
    or 1 hidden layers."""

    def __init__(self, ctx, seed=1, handle=None, hidden_layers=None):
        self.ctx = ctx
        self._lib = load()
        if handle is None:
            h = ctypes.c_void_p()
            layers = DEFAULT_LAYERS if hidden_layers is None else int(hidden_layers)
            check(self._lib.cg_mlp_create_layers(ctx.handle, int(seed), layers, ctypes.byref(h)),
                  "cg_mlp_create_layers")
            handle = h
        self.handle = handle

    @property
    def hidden_layers(self):
        return int(self._lib.cg_mlp_hidden_layers(self.handle))

    def copy_config(self, other):
        """Take another model's configuration (features, normalisation, cone)."""
        c = other.config
        check(self._lib.cg_mlp_configure(self.handle, ctypes.byref(c)), "cg_mlp_configure")

    @classmethod
    def load(cls, ctx, path):
        h = ctypes.c_void_p()
        check(load().cg_mlp_load(ctx.handle, os.fsencode(path), ctypes.byref(h)), "cg_mlp_load")
        return cls(ctx, handle=h)

    def save(self, path):
        check(self._lib.cg_mlp_save(self.handle, os.fsencode(path)), "cg_mlp_save")

    def close(self):
        if self.handle:
            self._lib.cg_mlp_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- configuration --
    @property
    def config(self):
        c = _lib.cg_mlp_config()
        check(self._lib.cg_mlp_get_config(self.handle, ctypes.byref(c)), "cg_mlp_get_config")
        return c

    def configure(self, **kw):
        c = self.config
        for k, v in kw.items():
            if k in ("mean", "stddev", "feature_min", "feature_max"):
                getattr(c, k)[:] = [float(x) for x in v]
            else:
                setattr(c, k, v)
        check(self._lib.cg_mlp_configure(self.handle, ctypes.byref(c)), "cg_mlp_configure")

    def configure_for(self, volume, shader):
        """Bind the model to a volume resolution and an exact-cone setting."""
        p = shader.params()
        lb = int(math.floor(math.log2(max(1.0, 2.0 * p.cone_min_radius))))
        self.configure(base_level=lb, initial_height=p.cone_initial_height,
                       dimension=volume.dimension, sun_steps=p.sun_steps,
                       cone_half_angle=p.cone_half_angle,
                       cone_initial_height=p.cone_initial_height,
                       cone_min_radius=p.cone_min_radius, lod_offset=p.lod_offset)

    # -- parameters --
    def get_params(self):
        p = np.empty(N_PARAMS, np.float32)
        m = np.empty(N_PARAMS, np.float32)
        v = np.empty(N_PARAMS, np.float32)
        step = ctypes.c_int()
        check(self._lib.cg_mlp_get_params(self.handle, _fp(p), _fp(m), _fp(v), ctypes.byref(step)),
              "cg_mlp_get_params")
        return p, m, v, int(step.value)

    def set_params(self, params, m=None, v=None, step=0):
        params = np.ascontiguousarray(params, np.float32)
        mm = None if m is None else _fp(np.ascontiguousarray(m, np.float32))
        vv = None if v is None else _fp(np.ascontiguousarray(v, np.float32))
        check(self._lib.cg_mlp_set_params(self.handle, _fp(params), mm, vv, int(step)),
              "cg_mlp_set_params")

    # -- compute --
    def features(self, volume, positions, direction):
        pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
        out = np.empty((pos.shape[0], N_FEATURES), np.float32)
        d = (ctypes.c_float * 3)(*[float(x) for x in direction])
        check(self._lib.cg_mlp_features(volume.handle, self.handle,
                                        pos.ctypes.data_as(ctypes.c_void_p), pos.shape[0], d,
                                        out.ctypes.data_as(ctypes.c_void_p), 0, None),
              "cg_mlp_features")
        return out

    def infer(self, features):
        f = np.ascontiguousarray(features, np.float32).reshape(-1, N_FEATURES)
        out = np.empty((f.shape[0],), np.float32)
        check(self._lib.cg_mlp_infer(self.handle, f.ctypes.data_as(ctypes.c_void_p), f.shape[0],
                                     out.ctypes.data_as(ctypes.c_void_p), 0, None),
              "cg_mlp_infer")
        return out

    def gradient(self, features, tau, sigma):
        f = np.ascontiguousarray(features, np.float32).reshape(-1, N_FEATURES)
        t = np.ascontiguousarray(tau, np.float32).reshape(-1)
        g = np.empty(N_PARAMS, np.float32)
        loss = ctypes.c_float()
        check(self._lib.cg_mlp_gradient(self.handle, f.ctypes.data_as(ctypes.c_void_p),
                                        t.ctypes.data_as(ctypes.c_void_p), f.shape[0],
                                        float(sigma), _fp(g), ctypes.byref(loss), 0),
              "cg_mlp_gradient")
        return g, float(loss.value)

    def train(self, features, tau, steps, batch=16384, lr=1e-3, sigma=2.0, seed=1,
              beta1=0.9, beta2=0.999, eps=1e-8, separate_adam=False):
        """Train on host arrays (uploaded once) and return the per-step loss.
        separate_adam: run Adam as its own launch even where it fits in the
        training launch (identical results)."""
        from . import DeviceBuffer
        f = np.ascontiguousarray(features, np.float32).reshape(-1, N_FEATURES)
        t = np.ascontiguousarray(tau, np.float32).reshape(-1)
        df = DeviceBuffer(f.nbytes)
        dt = DeviceBuffer(t.nbytes)
        df.upload(f)
        dt.upload(t)
        tp = _lib.cg_train_params()
        self._lib.cg_train_params_default(ctypes.byref(tp))
        tp.steps, tp.batch, tp.lr, tp.sigma, tp.seed = int(steps), int(batch), lr, sigma, seed
        tp.beta1, tp.beta2, tp.eps = beta1, beta2, eps
        tp.separate_adam = 1 if separate_adam else 0
        losses = np.empty(max(1, int(steps)), np.float32)
        check(self._lib.cg_mlp_train(self.handle, df.ptr, dt.ptr, f.shape[0], ctypes.byref(tp),
                                     _fp(losses)), "cg_mlp_train")
        df.free()
        dt.free()
        return losses[:steps]

    def fit_normalization(self, features, tau, margin=0.05):
        """Input mean/stddev, trusted range (observed range widened by `margin`
        of its span) and the output scale from a training set."""
        f = np.asarray(features, np.float64)
        mu = f.mean(axis=0)
        sd = f.std(axis=0)
        sd[sd < 1e-6] = 1.0
        lo, hi = f.min(axis=0), f.max(axis=0)
        span = np.maximum(hi - lo, 1e-6)
        tau_scale = float(max(np.std(tau), 1e-3))
        self.configure(mean=mu, stddev=sd, feature_min=lo - margin * span,
                       feature_max=hi + margin * span, tau_scale=tau_scale)


def march_samples(volume, shader, camera, capacity=4 << 20):
    """Contributing view samples of one view (positions in level-0 voxels, weights)."""
    lib = load()
    pos = np.empty((capacity, 3), np.float32)
    w = np.empty((capacity,), np.float32)
    n = ctypes.c_int()
    p = shader.params()
    c = camera._c()
    check(lib.cg_march_samples(volume.ctx.handle, volume.handle, ctypes.byref(c), ctypes.byref(p),
                               _fp(pos), _fp(w), capacity, ctypes.byref(n)), "cg_march_samples")
    k = min(int(n.value), capacity)
    return pos[:k], w[:k]


def training_set(ctx, shader, samples=4_000_000, scenes=16, dim=256, mips=8, fmt=None,
                 views_per_scene=4, view_size=(480, 270), seed=1000, mlp=None,
                 hidden_layers=None):
    """(features, tau, model) drawn from the renderer's view samples over
    training scenes (seeds seed .. seed + scenes - 1, disjoint from evaluation
    seeds); a new model (hidden_layers deep) is created unless one is given."""
    import cloudgb
    fmt = cloudgb.FORMAT_BF16_FP16 if fmt is None else fmt
    rng = scene.SplitMix64(seed)
    per_scene = int(math.ceil(samples / scenes))
    feats, taus = [], []
    for k in range(scenes):
        u = rng.uniform(4)
        count = int(round(math.exp(math.log(64) + u[0] * (math.log(4096) - math.log(64)))))
        rscale = 0.5 + 0.5 * u[1]
        pos, rad, den = scene.billboards(seed + 1 + k, count, radius_scale=rscale)
        # sun within ~30 degrees of the workload sun
        base = np.asarray(configs.SUN_DIRECTION, np.float64)
        base /= np.linalg.norm(base)
        # the first scene keeps the workload sun so the feature range covers it
        jitter = rng.on_unit_sphere(1)[0] * 0.5 * u[2]
        sd = base + (jitter if k > 0 else 0.0)
        sd /= np.linalg.norm(sd)
        vol = cloudgb.CloudVolume(dim, configs.VOLUME_BOUNDS, configs.VOLUME_POSITION, mips,
                                  fmt=fmt, ctx=ctx)
        vol.set_billboards(pos, rad, den)
        vol.update()
        sun = cloudgb.Sun(tuple(sd), *configs.PLAIN_1080P["sun_map"])
        cloudgb.VoxelizeShader().voxelize(vol, sun)
        if mlp is None:
            mlp = SunMLP(ctx, hidden_layers=hidden_layers)
            mlp.configure_for(vol, shader)
        eyes = scene.orbit_cameras(seed + 101 + k, views_per_scene)
        P, Wt = [], []
        for e in eyes:
            cam = cloudgb.Camera(e, (0.5, 0.5, 0.5), width=view_size[0], height=view_size[1])
            p, w = march_samples(vol, shader, cam)
            P.append(p)
            Wt.append(w)
        P = np.concatenate(P)
        Wt = np.concatenate(Wt).astype(np.float64)
        if P.shape[0] == 0:
            vol.close()
            continue
        # keep samples with probability proportional to their weight
        prob = Wt / Wt.sum()
        sel_rng = np.random.default_rng(seed * 7919 + k)
        take = min(per_scene, P.shape[0])
        idx = sel_rng.choice(P.shape[0], size=take, replace=True, p=prob)
        p = P[idx]
        tau = shader.traceCone(vol, p, sun.direction)
        f = mlp.features(vol, p, sun.direction)
        feats.append(f)
        taus.append(tau)
        vol.close()
    return np.concatenate(feats), np.concatenate(taus), mlp


def train_surrogate(ctx, shader, samples=4_000_000, steps=20000, batch=16384, lr=1e-3,
                    scenes=16, seed=1000, dim=256, mips=8, hidden_layers=None):
    """Generate the training set, fit the normalisation and train; returns
    (model, per-step loss)."""
    f, tau, mlp = training_set(ctx, shader, samples=samples, scenes=scenes, dim=dim, mips=mips,
                               seed=seed, hidden_layers=hidden_layers)
    mlp.fit_normalization(f, tau)
    losses = mlp.train(f, tau, steps, batch=batch, lr=lr, sigma=shader.densityScale, seed=seed)
    return mlp, losses
