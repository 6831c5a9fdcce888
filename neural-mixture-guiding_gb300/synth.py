"""Seeded synthetic inputs with the shapes and distributions of the guiding
step's workloads. The reference measures this path on rendered scenes, whose
data is not part of this project; these generators stand in for them.

* mixture_batch  -- raw network outputs of K-lobe mixtures, 4 uniforms per
  query and one KL training record per query (mixture kernels only).
* wavefront      -- shading queries (position, outgoing direction, normal,
  roughness) of one 1920x1080 bounce: 70% of positions on 64 random planes,
  30% uniform in the unit cube.
* train_field / train_batch -- a 16^3-cell ground-truth radiance field, each
  cell a 4-lobe vMF mixture, and training records drawn from it.

All arrays are float32 numpy, row-major, in the layouts of the C ABI
(include/nmg.h). numpy's PCG64 streams are platform-independent, so the same
seed gives the same inputs on every host.
"""
import math

import numpy as np

INV_4PI = 1.0 / (4.0 * math.pi)


def round16(x):
    return (x + 15) // 16 * 16


def uniform_sphere(rng, shape):
    u = rng.random(shape + (2,))
    z = 1.0 - 2.0 * u[..., 0]
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = 2.0 * math.pi * u[..., 1]
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=-1)


def _logit(p):
    p = np.clip(p, 1e-6, 1.0 - 1e-6)
    return np.log(p / (1.0 - p))


def cart_to_sph(v):
    v = v / np.linalg.norm(v, axis=-1, keepdims=True)
    theta = np.arccos(np.clip(v[..., 2], -1.0, 1.0))
    phi = np.arctan2(v[..., 1], v[..., 0])
    phi = np.where(phi < 0, phi + 2.0 * math.pi, phi)
    return theta, phi


def sph_to_cart(theta, phi):
    st = np.sin(theta)
    return np.stack([st * np.cos(phi), st * np.sin(phi), np.cos(theta)], axis=-1)


def _activate(raw, K):
    """FP64 activation of raw outputs [n, >=4K] -> weights, kappa, mu [n,K,3]."""
    r = raw[:, :4 * K].astype(np.float64).reshape(-1, K, 4)
    lam = np.exp(np.clip(r[..., 0], -10, 15))
    kap = np.exp(np.clip(r[..., 1], -10, 15))
    th = math.pi / (1.0 + np.exp(-r[..., 2]))
    ph = 2.0 * math.pi / (1.0 + np.exp(-r[..., 3]))
    w = lam / lam.sum(axis=1, keepdims=True)
    return w, kap, sph_to_cart(th, ph)


def vmf_pdf(kap, mu, wi):
    """Mixture-free vMF pdf, kap [..., K], mu [..., K, 3], wi [..., 3]."""
    c = np.einsum("...kj,...j->...k", mu, wi)
    k = np.maximum(kap, 1e-12)
    val = k * np.exp(k * np.minimum(0.0, c - 1.0)) / (2.0 * math.pi * -np.expm1(-2.0 * k))
    return np.where(kap < 1e-5, INV_4PI, val)


def _frame(n):
    a = np.abs(n)
    xm = ((a[:, 0] - a[:, 1]) < 0) & ((a[:, 0] - a[:, 2]) < 0)
    ym = (~xm) & ((a[:, 1] - a[:, 2]) < 0)
    zm = ~(xm | ym)
    e = np.stack([xm, ym, zm], axis=-1).astype(np.float64)
    t = np.cross(n, e)
    t /= np.linalg.norm(t, axis=-1, keepdims=True)
    b = np.cross(n, t)
    b /= np.linalg.norm(b, axis=-1, keepdims=True)
    return t, b


def sample_vmf(rng, kap, mu):
    """One sample per row from vMF(kap[i], mu[i])."""
    n = kap.shape[0]
    u = rng.random((n, 2))
    k = np.maximum(kap, 1e-6)
    ct = 1.0 + np.log1p(-u[:, 0] + np.exp(-2.0 * k) * u[:, 0]) / k
    st = np.sqrt(np.maximum(0.0, 1.0 - ct * ct))
    ph = 2.0 * math.pi * u[:, 1]
    t, b = _frame(mu)
    local = np.stack([np.cos(ph) * st, np.sin(ph) * st, ct], axis=-1)
    return t * local[:, :1] + b * local[:, 1:2] + mu * local[:, 2:3]


def sample_mixture(rng, w, kap, mu):
    n, K = w.shape
    cdf = np.cumsum(w, axis=1)
    u = rng.random(n)
    lobe = np.minimum((u[:, None] >= cdf).sum(axis=1), K - 1)
    idx = np.arange(n)
    return sample_vmf(rng, kap[idx, lobe], mu[idx, lobe])


def mixture_batch(n, K=8, seed=7272, selection=False, stride=None):
    """Mixture-only workload: raw outputs, uniforms and KL training records.

    raw [n, stride]: per lobe (lambda, kappa, theta, phi) raw logits; lambda
    ~ N(0,1), kappa = 10^U(-1,3) mapped through log, mean uniform on the
    sphere mapped through logit(theta/pi), logit(phi/2pi). With selection an
    extra selection logit ~ N(0,1) follows the lobes.
    u4 [n, 4]: (u_guide, u_lobe, u_dir0, u_dir1) in [0,1).
    rec [n, 6 or 7]: GuidedOutput {theta, phi, L_r, L_g, L_b, wiPdf[, bsdfPdf]};
    the direction is drawn 50% from the query's own mixture, 50% uniformly,
    wiPdf is the pdf of that draw and L/wiPdf ~ lognormal(0, 1.5).
    """
    rng = np.random.default_rng(seed)
    nout = 4 * K + (1 if selection else 0)
    stride = stride or round16(nout)
    raw = np.zeros((n, stride), np.float32)
    lam = rng.standard_normal((n, K))
    kap = 10.0 ** rng.uniform(-1.0, 3.0, (n, K))
    mu = uniform_sphere(rng, (n, K))
    th, ph = cart_to_sph(mu)
    r = raw[:, :4 * K].reshape(n, K, 4)
    r[..., 0] = lam
    r[..., 1] = np.log(kap)
    r[..., 2] = _logit(th / math.pi)
    r[..., 3] = _logit(ph / (2.0 * math.pi))
    raw[:, :4 * K] = r.reshape(n, 4 * K)
    if selection:
        raw[:, 4 * K] = rng.standard_normal(n)
    u4 = rng.random((n, 4), dtype=np.float32)

    w, kk, mm = _activate(raw, K)
    own = sample_mixture(rng, w, kk, mm)
    uni = uniform_sphere(rng, (n,))
    pick = rng.random(n) < 0.5
    wi = np.where(pick[:, None], own, uni)
    q = (w * vmf_pdf(kk, mm, wi)).sum(axis=1)
    wi_pdf = 0.5 * q + 0.5 * INV_4PI
    weight = rng.lognormal(0.0, 1.5, n)
    Li = weight * wi_pdf
    dth, dph = cart_to_sph(wi)
    cols = [dth, dph, 0.8 * Li, 1.0 * Li, 1.2 * Li, wi_pdf]
    if selection:
        cols.append(np.full(n, INV_4PI))
    rec = np.stack(cols, axis=-1).astype(np.float32)
    return raw, u4, rec


def _plane_points(rng, n, n_planes=64, seed_planes=None):
    prng = np.random.default_rng(seed_planes) if seed_planes is not None else rng
    pn = uniform_sphere(prng, (n_planes,))
    off = np.einsum("pj,pj->p", pn, prng.random((n_planes, 3)))
    p = rng.random((n, 3))
    k = rng.integers(0, n_planes, n)
    d = np.einsum("nj,nj->n", p, pn[k]) - off[k]
    return np.clip(p - d[:, None] * pn[k], 0.0, 1.0)


def wavefront(n, seed=7272):
    """Shading queries of one bounce: dict of pos/wo/normal [n,3], rough [n],
    u4 [n,4] (float32) and the scene box aabb [6] = unit cube."""
    rng = np.random.default_rng(seed)
    n_pl = int(round(0.7 * n))
    pos = np.concatenate([_plane_points(rng, n_pl, seed_planes=seed + 1), rng.random((n - n_pl, 3))])
    pos = pos[rng.permutation(n)]
    return {
        "pos": pos.astype(np.float32),
        "wo": uniform_sphere(rng, (n,)).astype(np.float32),
        "normal": uniform_sphere(rng, (n,)).astype(np.float32),
        "rough": rng.random(n, dtype=np.float32),
        "u4": rng.random((n, 4), dtype=np.float32),
        "aabb": np.array([0, 0, 0, 1, 1, 1], np.float32),
    }


class TrainField:
    """Ground-truth radiance field: 16^3 cells, each a 4-lobe vMF mixture with
    kappa log-uniform on [1, 200] and uniform mean directions."""

    def __init__(self, seed=7272, cells=16, lobes=4):
        rng = np.random.default_rng(seed + 17)
        self.cells = cells
        nc = cells ** 3
        self.w = rng.random((nc, lobes)) + 0.1
        self.w /= self.w.sum(axis=1, keepdims=True)
        self.kap = 10.0 ** rng.uniform(0.0, math.log10(200.0), (nc, lobes))
        self.mu = uniform_sphere(rng, (nc, lobes))

    def cell(self, pos):
        c = np.clip((pos * self.cells).astype(np.int64), 0, self.cells - 1)
        return (c[:, 0] * self.cells + c[:, 1]) * self.cells + c[:, 2]

    def density(self, cell, wi):
        return (self.w[cell] * vmf_pdf(self.kap[cell], self.mu[cell], wi)).sum(axis=1)

    def sample(self, rng, cell):
        return sample_mixture(rng, self.w[cell], self.kap[cell], self.mu[cell])


def featurize(q, input_mode=1):
    """Network input rows from shading data (train.cu:174-191 for mode 0;
    mode 1 encodes the normal as (n+1)/2 for its spherical harmonics)."""
    aabb = q["aabb"].astype(np.float32)
    mn, mx = aabb[:3], aabb[3:]
    infl = np.float32(np.linalg.norm(mx - mn) * 0.005)
    lo, hi = mn - infl, mx + infl
    c, d = (lo + hi) / 2, hi - lo
    p = 0.5 + (q["pos"] - c) / d
    wo = q["wo"] / np.linalg.norm(q["wo"], axis=1, keepdims=True)
    cols = [p, (wo + 1.0) * 0.5]
    nrm = q["normal"] / np.linalg.norm(q["normal"], axis=1, keepdims=True)
    if input_mode == 0:
        th, ph = cart_to_sph(nrm.astype(np.float64))
        cols.append(np.stack([th / math.pi, ph / (2 * math.pi)], axis=-1))
    else:
        cols.append((nrm + 1.0) * 0.5)
    cols.append((1.0 - np.exp(-q["rough"]))[:, None])
    return np.concatenate(cols, axis=1).astype(np.float32)


def train_batch(field, n, seed=7272, input_mode=1, selection=False):
    """Training records drawn from the field: (inputs [n, 9|10] network input
    rows, records [n, 6|7] GuidedOutput)."""
    rng = np.random.default_rng(seed)
    q = wavefront(n, seed=seed + 1000)
    cell = field.cell(q["pos"].astype(np.float64))
    own = field.sample(rng, cell)
    uni = uniform_sphere(rng, (n,))
    pick = rng.random(n) < 0.5
    wi = np.where(pick[:, None], own, uni)
    dens = field.density(cell, wi)
    wi_pdf = 0.5 * dens + 0.5 * INV_4PI
    L = dens * rng.lognormal(0.0, 0.5, n)
    th, ph = cart_to_sph(wi)
    cols = [th, ph, 0.8 * L, 1.0 * L, 1.2 * L, wi_pdf]
    if selection:
        cols.append(np.full(n, INV_4PI))
    return featurize(q, input_mode), np.stack(cols, axis=-1).astype(np.float32)


class TorchTrainSource:
    """Fresh training batches drawn on the GPU from a TrainField, one per call,
    as a renderer would record them each frame (the same distributions as
    train_batch: 70% of positions on the 64 planes of `wavefront`, 30% uniform;
    wi 50% from the cell's mixture, 50% uniform; radiance = density x
    lognormal(0, 0.5); wiPdf the pdf of that draw). Returns float32 CUDA
    tensors (inputs [n, 10], records [n, 6|7]) for input mode 1."""

    def __init__(self, field, seed=7272, device="cuda", plane_seed=None):
        import torch
        self.torch = torch
        self.dev = device
        self.gen = torch.Generator(device=device)
        self.gen.manual_seed(seed)
        self.cells = field.cells
        t = lambda a: torch.as_tensor(np.asarray(a, np.float64), device=device)
        self.w, self.kap, self.mu = t(field.w), t(field.kap), t(field.mu)
        # the planes of wavefront(n, s) come from seed s + 1: plane_seed = s + 1 puts the training
        # records on the same surfaces as that wavefront's queries
        prng = np.random.default_rng(seed + 1 if plane_seed is None else plane_seed)
        pn = uniform_sphere(prng, (64,))
        self.pn = t(pn)
        self.off = t(np.einsum("pj,pj->p", pn, prng.random((64, 3))))
        infl = math.sqrt(3.0) * 0.005  # the unit box inflated by 0.5% of its diagonal (train.h:173-177)
        self.lo, self.size = -infl, 1.0 + 2.0 * infl

    def _rand(self, *shape):
        return self.torch.rand(*shape, generator=self.gen, device=self.dev, dtype=self.torch.float64)

    def _sphere(self, n):
        torch = self.torch
        u = self._rand(n, 2)
        z = 1.0 - 2.0 * u[:, 0]
        r = torch.sqrt(torch.clamp(1.0 - z * z, min=0.0))
        ph = 2.0 * math.pi * u[:, 1]
        return torch.stack([r * torch.cos(ph), r * torch.sin(ph), z], dim=-1)

    def density(self, cell, wi):
        torch = self.torch
        k = self.kap[cell]
        c = (self.mu[cell] * wi[:, None, :]).sum(-1)
        v = k * torch.exp(k * torch.clamp(c - 1.0, max=0.0)) / (2.0 * math.pi * -torch.expm1(-2.0 * k))
        return (self.w[cell] * v).sum(-1)

    def __call__(self, n, selection=False):
        torch = self.torch
        n_pl = int(round(0.7 * n))
        p = self._rand(n, 3)
        k = torch.randint(0, 64, (n_pl,), generator=self.gen, device=self.dev)
        d = (p[:n_pl] * self.pn[k]).sum(-1) - self.off[k]
        p[:n_pl] = torch.clamp(p[:n_pl] - d[:, None] * self.pn[k], 0.0, 1.0)
        ci = torch.clamp((p * self.cells).long(), 0, self.cells - 1)
        cell = (ci[:, 0] * self.cells + ci[:, 1]) * self.cells + ci[:, 2]
        # wi from the cell's mixture: lobe by CDF, vMF by inversion
        lobe = torch.multinomial(self.w[cell], 1, generator=self.gen).squeeze(1)
        kap = self.kap[cell, lobe]
        mu = self.mu[cell, lobe]
        u = self._rand(n, 2)
        ct = 1.0 + torch.log1p(u[:, 0] * torch.expm1(-2.0 * kap)) / kap
        st = torch.sqrt(torch.clamp(1.0 - ct * ct, min=0.0))
        ph = 2.0 * math.pi * u[:, 1]
        a = torch.where(mu[:, 2:3].abs() < 0.9, torch.tensor([0.0, 0.0, 1.0], device=self.dev, dtype=torch.float64),
                        torch.tensor([1.0, 0.0, 0.0], device=self.dev, dtype=torch.float64))
        t1 = torch.nn.functional.normalize(torch.cross(mu, a, dim=-1), dim=-1)
        t2 = torch.cross(mu, t1, dim=-1)
        own = t1 * (st * torch.cos(ph))[:, None] + t2 * (st * torch.sin(ph))[:, None] + mu * ct[:, None]
        pick = self._rand(n) < 0.5
        wi = torch.where(pick[:, None], own, self._sphere(n))
        wi = torch.nn.functional.normalize(wi, dim=-1)
        dens = self.density(cell, wi)
        L = dens * torch.exp(0.5 * torch.randn(n, generator=self.gen, device=self.dev, dtype=torch.float64))
        th = torch.acos(torch.clamp(wi[:, 2], -1.0, 1.0))
        phi = torch.atan2(wi[:, 1], wi[:, 0])
        phi = torch.where(phi < 0, phi + 2.0 * math.pi, phi)
        cols = [th, phi, 0.8 * L, L, 1.2 * L, 0.5 * dens + 0.5 * INV_4PI]
        if selection:
            cols.append(torch.full_like(th, INV_4PI))
        rec = torch.stack(cols, dim=-1).float()
        x = torch.cat([0.5 + (p - (self.lo + self.size / 2)) / self.size,
                       (self._sphere(n) + 1.0) * 0.5,   # wo
                       (self._sphere(n) + 1.0) * 0.5,   # normal
                       (1.0 - torch.exp(-self._rand(n)))[:, None]], dim=1).float()
        return x.contiguous(), rec.contiguous()
