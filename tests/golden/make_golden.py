"""Writes tests/golden/mixture_golden.npz from the REFERENCE'S OWN mixture code.

Run in a checkout where the reference exists (it compiles
oracle/_ref/libnmgref.so through oracle/build_ref.sh):

    python tests/golden/make_golden.py

Inputs are seeded synthetic mixtures (neural-mixture-guiding_gb300/synth.py)
plus hand-written edge rows: clamped lambda/kappa logits, lobe means at the
poles, uniforms at 0 and just below 1, directions and normals on the axes.
Outputs come from the reference's distribution.h / vmf.h / train.h compiled
on the host (K = 8, the reference's compile-time lobe count):
  sample  -- MixedSG(raw).sample() + pdf(), with and without applyCosineLobe
  pdf     -- MixedSG(raw).pdf(wi) at given directions
  loss    -- the reference's compute_dL_doutput_divergence kernel
             (train.cu:69-124) run on the host, with __half raw outputs and
             gradients.
It also writes tests/golden/train_cu_golden.npz from the reference's
generate_training_data and generate_inference_data kernels (train_cu()).
"""
import importlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402

synth = importlib.import_module("neural-mixture-guiding_gb300.synth")

K = 8
N_RANDOM = 1024
SEED = 7272


def edge_rows(rng):
    rows, u4s = [], []
    base_raw, base_u, _ = synth.mixture_batch(64, K, seed=SEED + 99)
    for i in range(64):
        r = base_raw[i].copy()
        u = base_u[i].copy()
        lobe = i % K
        kind = i // K
        if kind == 0:
            r[4 * lobe + 0] = 20.0   # lambda logit above the exp clamp
        elif kind == 1:
            r[4 * lobe + 0] = -20.0  # below the clamp
            r[4 * lobe + 1] = -20.0  # kappa -> exp(-10)
        elif kind == 2:
            r[4 * lobe + 1] = 9.0    # kappa ~ 8100
        elif kind == 3:
            r[4 * lobe + 2] = 20.0   # theta -> pi (south pole)
            r[4 * lobe + 3] = -20.0  # phi -> 0
        elif kind == 4:
            r[4 * lobe + 2] = -20.0  # theta -> 0 (north pole)
        elif kind == 5:
            u[1] = 0.0
            u[2] = 0.0
        elif kind == 6:
            u[1] = np.float32(0.99999994)
            u[2] = np.float32(0.99999994)
            u[3] = np.float32(0.99999994)
        else:
            r[0:4 * K:4] = 0.0       # equal weights: CDF boundaries at k/8
            u[1] = np.float32(lobe / K)
        rows.append(r)
        u4s.append(u)
    return np.array(rows, np.float32), np.array(u4s, np.float32)


def main():
    if O.ref_lib() is None:
        raise SystemExit("reference checkout not available; cannot regenerate golden vectors")
    rng = np.random.default_rng(SEED)
    raw, u4, rec = synth.mixture_batch(N_RANDOM, K, seed=SEED)
    er, eu = edge_rows(rng)
    raw = np.concatenate([raw, er])
    u4 = np.concatenate([u4, eu])
    n = raw.shape[0]
    _, _, erec = synth.mixture_batch(64, K, seed=SEED + 5)
    rec = np.concatenate([rec, erec])
    axes = np.array([[0, 0, 1], [0, 0, -1], [1, 0, 0], [0, 1, 0], [0, -1, 0], [-1, 0, 0]], np.float32)
    cosn = synth.uniform_sphere(rng, (n,)).astype(np.float32)
    cosn[:6] = axes
    wi = synth.uniform_sphere(rng, (n,)).astype(np.float32)
    wi[6:12] = axes

    d, p, lb = O.ref_mixture_sample(raw, u4)
    dc, pc, lbc = O.ref_mixture_sample(raw, u4, cosn)
    pe = O.ref_mixture_pdf(raw, wi)
    pec = O.ref_mixture_pdf(raw, wi, cosn)
    g, loss = O.ref_loss_grad(raw, rec, 128.0)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "mixture_golden.npz")
    np.savez_compressed(out, K=K, raw=raw, u4=u4, rec=rec, cosn=cosn, wi=wi, dir=d, pdf=p, lobe=lb, dir_cos=dc,
                        pdf_cos=pc, lobe_cos=lbc, pdf_eval=pe, pdf_eval_cos=pec, grad=g, loss=loss,
                        loss_scale=np.float32(128.0))
    print("wrote", out, "rows", n, "bytes", os.path.getsize(out))


# ---------------------------------------------------------------------------
# train_cu_golden.npz: the reference's own train.cu kernels (compiled as host
# functions by oracle/ref_shim.cu) on seeded inputs.
#   records   -- generate_training_data (train.cu:14-67) over a
#                GuidedPixelStateBuffer of 8 depths: delta vertices, thp below
#                and exactly at M_EPSILON = 1e-5, NaN position / direction /
#                outgoing direction / pdf / MIS weight / radiance, NaN and Inf
#                bsdfVal, zero pdfs, a training-pixel grid running off the image
#   featurize -- generate_inference_data (train.cu:174-191) over a
#                ScatterRayQueue (soac-generated SOA<ScatterRayWorkItem>):
#                positions inside, on and outside the box, non-unit outgoing
#                directions, normals on the axes and poles; the queue's own
#                field arrays are stored with the rows
# ---------------------------------------------------------------------------
REC_RES = (29, 23)
REC_OFFSET, REC_STRIDE = (1, 2), (3, 2)
REC_TRAIN_RES = (10, 12)  # the grid's last row and column fall outside the image
REC_AABB = (-2.0, -1.5, -2.5, 3.0, 3.5, 2.0)
DEPTH = 8


def record_inputs(seed):
    rng = np.random.default_rng(seed)
    n = REC_RES[0] * REC_RES[1]
    rec = {}

    def ang(m):
        return np.stack([rng.uniform(0, np.pi, m), rng.uniform(0, 2 * np.pi, m)], 1).astype(np.float32)

    per = []
    for _ in range(DEPTH):
        r = {}
        thp = rng.uniform(0, 1, (n, 3)).astype(np.float32)
        thp[rng.random((n, 3)) < 0.05] = 5e-6
        thp[rng.random((n, 3)) < 0.05] = np.float32(1e-5)  # exactly M_EPSILON: not above it
        r["thp"] = thp
        L = rng.lognormal(0, 1, (n, 3)).astype(np.float32)
        L[rng.random(n) < 0.01, 1] = np.nan
        r["L"] = L
        pos = rng.uniform(-2.5, 3.5, (n, 3)).astype(np.float32)
        pos[rng.random(n) < 0.01, 0] = np.nan
        r["pos"] = pos
        d = ang(n)
        d[rng.random(n) < 0.01, 1] = np.nan
        r["dir"] = d
        wp = rng.uniform(0.01, 2, n).astype(np.float32)
        wp[rng.random(n) < 0.02] = 0.0
        wp[rng.random(n) < 0.01] = np.nan
        r["wi_pdf"] = wp
        r["bsdf_pdf"] = rng.uniform(0.01, 2, n).astype(np.float32)
        mw = rng.uniform(0, 1, n).astype(np.float32)
        mw[rng.random(n) < 0.01] = np.nan
        r["mis_weight"] = mw
        r["delta"] = (rng.random(n) < 0.1).astype(np.uint8)
        bv = rng.uniform(0, 1, (n, 3)).astype(np.float32)
        bv[rng.random(n) < 0.02, 0] = np.nan   # kept by the reference: NaN only in the stored radiance
        bv[rng.random(n) < 0.02, 2] = np.inf
        r["bsdf_val"] = bv
        wo = ang(n)
        wo[rng.random(n) < 0.015, 0] = np.nan  # NaN warped outgoing direction: dropped
        wo[rng.random(n) < 0.015, 1] = np.nan
        r["wo"] = wo
        r["normal"] = ang(n)
        r["roughness"] = rng.uniform(0, 1, n).astype(np.float32)
        per.append(r)
    for k in per[0]:
        rec[k] = np.stack([r[k] for r in per])
    cur = rng.integers(0, DEPTH + 1, n).astype(np.uint32)
    # pixels off the training grid are never read: zero them so the fixture compresses
    on = np.zeros(n, bool)
    for ty in range(REC_TRAIN_RES[1]):
        for tx in range(REC_TRAIN_RES[0]):
            px, py = tx * REC_STRIDE[0] + REC_OFFSET[0], ty * REC_STRIDE[1] + REC_OFFSET[1]
            if px < REC_RES[0] and py < REC_RES[1]:
                on[px + py * REC_RES[0]] = True
    for k in rec:
        rec[k][:, ~on] = 0
    cur[~on] = 0
    return rec, cur


def queue_inputs(seed, n=1024):
    rng = np.random.default_rng(seed)
    lo, hi = np.array(REC_AABB[:3], np.float32), np.array(REC_AABB[3:], np.float32)
    pos = rng.uniform(lo - 0.1, hi + 0.1, (n, 3)).astype(np.float32)
    pos[:8] = np.array([[x, y, z] for x in (lo[0], hi[0]) for y in (lo[1], hi[1]) for z in (lo[2], hi[2])])
    wo = synth.uniform_sphere(rng, (n,)).astype(np.float32) * rng.uniform(0.5, 2.0, (n, 1)).astype(np.float32)
    nrm = synth.uniform_sphere(rng, (n,)).astype(np.float32)
    axes = np.array([[0, 0, 1], [0, 0, -1], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0]], np.float32)
    nrm[8:14] = axes
    wo[14:20] = axes * 3.0
    rough = rng.uniform(0, 1, n).astype(np.float32)
    rough[20:22] = (0.0, 1.0)
    return pos, wo, nrm, rough


def train_cu():
    rec, cur = record_inputs(SEED + 11)
    recd = {k: [v[d] for d in range(DEPTH)] for k, v in rec.items()}
    x, out = O.ref_extract_records(recd, cur, REC_OFFSET, REC_STRIDE, REC_TRAIN_RES, REC_RES, REC_AABB)
    pos, wo, nrm, rough = queue_inputs(SEED + 12)
    fx, leaves = O.ref_featurize_queue(pos, wo, nrm, rough, REC_AABB)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "train_cu_golden.npz")
    np.savez_compressed(
        path, res=np.array(REC_RES, np.uint32), offset=np.array(REC_OFFSET, np.uint32),
        stride=np.array(REC_STRIDE, np.uint32), train_res=np.array(REC_TRAIN_RES, np.uint32),
        aabb=np.array(REC_AABB, np.float32), cur_depth=cur, **{"rec_" + k: v for k, v in rec.items()},
        rec_x=x, rec_out=out, q_pos=pos, q_wo=wo, q_normal=nrm, q_rough=rough, q_x=fx,
        soa_pos=leaves["pos"], soa_wo=leaves["wo"], soa_normal=leaves["normal"], soa_rough=leaves["roughness"])
    print("wrote", path, "records", len(x), "queries", len(fx), "bytes", os.path.getsize(path))


# ---------------------------------------------------------------------------
# tcnn_golden.npz: tiny-cuda-nn 1.7's own code (oracle/ref_tcnn_kernels.cu,
# oracle/ref_tcnn_layout.cu) on seeded inputs, for both network presets:
#   layout    -- GridEncodingTemplated's level offsets and parameter count
#   grid      -- kernel_grid features and kernel_grid_backward table gradients
#                for a table given by a fixed integer formula (table_values)
#   sh, oneblob -- kernel_sh (degrees 2 and 4) and kernel_one_blob_soa (4 bins)
#   adam      -- three EMA(Adam) steps (adam_step + full- and half-precision EMA)
#                with the reference's optimiser settings (base.json)
#   snapshot  -- Trainer::serialize + nlohmann to_msgpack of a small network's
#                parameters, as __half and as float
# ---------------------------------------------------------------------------
def table_values(n):
    """The grid table both the fixture and its tests use: ((i * 2654435761) mod 2^32) / 2^32 - 0.5."""
    i = np.arange(n, dtype=np.uint64)
    return (((i * np.uint64(2654435761)) % np.uint64(1 << 32)).astype(np.float64) / 2.0 ** 32 - 0.5).astype(np.float32)


SNAPSHOT_CONFIG = dict(grid_levels=2, grid_base_resolution=4)  # on NMG_PRESET_REFERENCE: 13,408 parameters


def grid_positions(rng, res0, n=256):
    pos = rng.random((n, 3)).astype(np.float32)
    pos[:8] = np.array([[x, y, z] for x in (0, 1) for y in (0, 1) for z in (0, 1)], np.float32)
    pos[8] = 0.5
    pos[9:12] = np.float32(1.0 / res0) * np.arange(1, 4, dtype=np.float32)[:, None]  # on level-0 vertices
    pos[12] = np.float32(np.nextafter(np.float32(1), np.float32(0)))
    return pos


def tcnn():
    nmg = importlib.import_module("neural-mixture-guiding_gb300")
    rng = np.random.default_rng(SEED + 21)
    out = {}
    for preset in (nmg.PRESET_HASHGRID, nmg.PRESET_REFERENCE):
        cfg = nmg.config(preset)
        tag = "hash" if preset == nmg.PRESET_HASHGRID else "dense"
        F, Lv = int(cfg.grid_features), int(cfg.grid_levels)
        offs, npar = O.ref_tcnn_grid_layout(F, Lv, cfg.grid_log2_hashmap, cfg.grid_base_resolution,
                                            cfg.grid_per_level_scale, cfg.grid_hash, cfg.grid_smoothstep)
        table = table_values(int(offs[-1]) * F)
        pos = grid_positions(rng, cfg.grid_base_resolution)
        args = (F, offs, cfg.grid_base_resolution, cfg.grid_per_level_scale, cfg.grid_hash, cfg.grid_smoothstep)
        feats = O.ref_tcnn_grid_forward(*args, table, pos)
        bpos = pos[:48]
        dl = rng.standard_normal((len(bpos), Lv * F)).astype(np.float32)
        g = O.ref_tcnn_grid_backward(*args, bpos, dl)
        nz = np.nonzero(g)[0].astype(np.int64)
        out.update({tag + "_offsets": offs, tag + "_n_params": np.int64(npar), tag + "_pos": pos,
                    tag + "_features": feats, tag + "_bwd_pos": bpos, tag + "_dl_dy": dl,
                    tag + "_grad_index": nz, tag + "_grad_value": g[nz]})
    d = synth.uniform_sphere(rng, (256,)).astype(np.float32)
    d[:6] = np.array([[0, 0, 1], [0, 0, -1], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0]], np.float32)
    x01 = ((d + 1) * 0.5).astype(np.float32)
    out["sh_in"] = x01
    out["sh2"] = O.ref_tcnn_sh(2, x01)
    out["sh4"] = O.ref_tcnn_sh(4, x01)
    ob = rng.random((256, 3)).astype(np.float32)
    ob[:6, 0] = (0.0, 0.25, 0.5, 0.75, np.nextafter(np.float32(1), np.float32(0)), 1.0)
    out["oneblob_in"] = ob
    out["oneblob4"] = O.ref_tcnn_oneblob(4, ob)
    # three optimiser steps on 4,096 parameters, the first 1,024 matrix weights; some non-matrix
    # gradients are exactly zero (those parameters keep their state)
    n, n_mat = 4096, 1024
    w0 = (rng.standard_normal(n) * 0.1).astype(np.float32)
    grads = []
    for _ in range(3):
        gg = (rng.standard_normal(n) * 4.0).astype(np.float16).astype(np.float32)
        gg[n_mat:][rng.random(n - n_mat) < 0.3] = 0.0
        grads.append(gg)
    for full in (True, False):
        st = {"w_full": w0.copy(), "w16": w0.astype(np.float16).astype(np.float32), "m": np.zeros(n, np.float32),
              "v": np.zeros(n, np.float32), "psteps": np.zeros(n, np.uint32),
              "ema16": np.zeros(n, np.float32), "ema_tmp": np.zeros(n, np.float32)}
        for k in range(3):
            O.ref_tcnn_adam_ema(st, grads[k], n_mat, k + 1, full_precision=full)
        key = "adam_full" if full else "adam_half"
        for name in ("w_full", "m", "v", "psteps", "ema16", "ema_tmp"):
            out[key + "_" + name] = st[name]
    out["adam_w0"] = w0
    out["adam_grads"] = np.stack(grads)
    out["adam_n_matrix"] = np.int64(n_mat)
    scfg = nmg.config(nmg.PRESET_REFERENCE, **SNAPSHOT_CONFIG)
    sn = int(nmg.config_info(scfg).n_params)
    sp = (table_values(sn) * np.float32(0.2)).astype(np.float32)
    out["snapshot_n_params"] = np.int64(sn)
    out["snapshot_half"] = np.frombuffer(O.ref_tcnn_snapshot(sp, "__half"), np.uint8)
    out["snapshot_float"] = np.frombuffer(O.ref_tcnn_snapshot(sp, "float"), np.uint8)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tcnn_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, "bytes", os.path.getsize(path))


if __name__ == "__main__":
    main()
    train_cu()
    tcnn()
