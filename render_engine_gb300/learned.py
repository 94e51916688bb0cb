"""The learned radiance cache in the frame loop (host side).

The network of include/rc_mlp.h stands where the per-point cache stands: every frame

1. the network's per-light radiance at every cache point is written into the context's cache
   buffer (rc_mlp_infer into rc_array_info(RC_A_LC), the cache's own layout);
2. the frame runs (rc_frame) with a method whose history is one frame long (nmax 1, `rays` rays
   per point), so that each point's cache value becomes this frame's one-bounce estimate
   A(hit) (Edir(hit) + L(hit)) with L(hit) the network's radiance at the hit point: paths the
   tracer itself generates, bootstrapped on the network as a neural radiance cache is;
3. `steps_per_frame` Adam steps (rc_mlp_train, loss-scaled) on `batch` random points each, with
   those estimates as targets (`event_steps` more in each of the `event_frames` frames that
   follow a state change).

The network's inputs per point are its position and normal in the state's geometry and
(albedo, direct light of lights 0..2) of that state, each light's direct light divided by a
constant, so a light switched off reaches the network through its input at once.  The value the cache serves (and whose error is measured) is the
network's output of step 1.  There is no counterpart in the reference: its bench A calls the
closed NRC library; this cache is compared with the reference's own per-point cache methods.
"""
from __future__ import annotations

import numpy as np

from . import methods as M
from . import mlp as MLP
from . import native as N
from . import scene as S

# The frame method of the learned cache: a one-frame history (alpha = 1), one ray per point.
LEARNED_METHOD = M.Method(name="learned cache", mode=0, nmax=1.0, budget=1.0)


class LearnedCache:
    """The learned cache over a context that has a scene loaded (at most three lights: the
    network's inputs carry the direct light of lights 0..2)."""

    def __init__(self, ctx: N.Context, data: bytes, stream: int, batch: int = 1 << 16, lr: float = 1e-2, seed: int = 1,
                 loss_scale: float = 0.0, steps_per_frame: int = 1, rays: float = 1.0, event_steps: int = 0,
                 event_frames: int = 0):
        import torch
        info = ctx.info()
        self.ctx, self.np, self.nl = ctx, info["np"], info["nl"]
        if self.nl > 3:
            raise ValueError("the learned cache takes scenes of at most three lights")
        self.lcs = (self.nl + 3) // 4 * 4
        sc = S.read(data)
        lo, hi = (0.0, 0.0, 0.0), (8.0, 4.0, 3.0)
        if sc.fmt == 3:
            lo = tuple(float(x) for x in sc.mesh["lo"])
            hi = tuple(float(a + b) for a, b in zip(sc.mesh["lo"], sc.mesh["ext"]))
        self.mlp = MLP.Mlp(box_lo=lo, box_hi=hi, n_out=self.nl, lr=lr, seed=seed, max_batch=batch, stream=stream,
                           loss_scale=loss_scale)
        self.batch = batch
        self.steps_per_frame = steps_per_frame
        # after a state change: event_steps more steps per frame for event_frames frames
        self.event_steps, self.event_frames = event_steps, event_frames
        self.last_state, self.boost_left = None, 0
        self.method = LEARNED_METHOD.replace(budget=float(rays))
        dev = torch.device("cuda", torch.cuda.current_device())
        # the direct light enters scaled by one constant per light (its largest mean over the
        # states), so that the inputs stay near 1 and a light off reads 0
        ed = [ctx.state_array(k, N.SA_EDIR).reshape(self.np, self.nl) for k in range(len(sc.states))]
        scale = np.maximum(np.max([e.mean(axis=0) for e in ed], axis=0), 1e-6).astype(np.float32)
        self.feat = []
        for k, st in enumerate(sc.states):
            p4 = np.zeros((self.np, 4), np.float32)
            n4 = np.zeros((self.np, 4), np.float32)
            a4 = np.zeros((self.np, 4), np.float32)
            p4[:, :3] = st.P
            n4[:, :3] = st.N
            a4[:, 0] = sc.A
            a4[:, 1:1 + self.nl] = ed[k] / scale
            self.feat.append(tuple(torch.from_numpy(x).to(dev) for x in (p4, n4, a4)))
        self.gen = torch.Generator(device=dev)
        self.gen.manual_seed(seed)
        self.dev = dev
        # one index buffer refilled every step: the training step's arguments stay the same, so
        # the library replays its captured graph of the step
        self.idx = torch.empty(batch, dtype=torch.int32, device=dev)

    def begin(self, state: int, seed: int):
        self.ctx.begin(self.method, state, seed)

    def pretrain(self, state: int, target, steps: int):
        """`steps` training steps on fixed per-point targets (a (Np, NL) CUDA tensor), e.g. a converged
        cache to start from."""
        import torch
        p4, n4, a4 = self.feat[state]
        for _ in range(steps):
            idx = torch.randint(0, self.np, (self.batch,), device=self.dev, generator=self.gen, dtype=torch.int32)
            self.mlp.train(p4, n4, a4, target, idx=idx)

    def predict(self, state: int):
        """The network's radiance into the context's cache buffer (what the cache serves)."""
        p4, n4, a4 = self.feat[state]
        self.mlp.infer_raw(p4, n4, a4, self.np, self.ctx.device_ptr(N.A_LC), self.lcs)

    def frame(self, state: int, predicted: bool = False):
        """One frame: predict (unless already done), trace and gather, train."""
        import torch
        if not predicted:
            self.predict(state)
        self.ctx.frame(state)
        if self.last_state is not None and state != self.last_state:
            self.boost_left = self.event_frames
        self.last_state = state
        steps = self.steps_per_frame
        if self.boost_left > 0:
            steps += self.event_steps
            self.boost_left -= 1
        p4, n4, a4 = self.feat[state]
        for _ in range(steps):
            torch.randint(0, self.np, (self.batch,), generator=self.gen, out=self.idx)
            self.mlp.train_raw(p4, n4, a4, self.ctx.device_ptr(N.A_LC), self.lcs, self.idx, self.batch)

    def close(self):
        self.mlp.close()
