"""CPU oracle for the guiding step -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package; it is the checker, never the thing measured or shipped.

Two libraries sit behind it:
  * oracle/_build/libnmg_oracle.so -- the scalar-templated C++ restatement
    (nmg_oracle.hpp, oracle_capi.cpp), FP64 and reference-order FP32;
  * oracle/_ref/libnmgref.so -- the reference's own mixture code compiled on
    the host by oracle/build_ref.sh (only where the reference checkout exists;
    used here to pin the restatement and to write tests/golden/).
"""
import ctypes as C
import os

import numpy as np

from . import build_oracle

_lib = None
_ref = None


class Opts(C.Structure):
    _fields_ = [("kappa_poly", C.c_int), ("expm1_norm", C.c_int), ("kappa_softplus", C.c_int),
                ("half_grad", C.c_int)]


def opts(kappa_poly=1, expm1_norm=0, kappa_softplus=0, half_grad=0):
    return Opts(kappa_poly, expm1_norm, kappa_softplus, half_grad)


class Net(C.Structure):
    _fields_ = [("input_mode", C.c_int), ("grid_hash", C.c_int), ("grid_levels", C.c_int),
                ("grid_feats", C.c_int), ("grid_log2_T", C.c_int), ("grid_base_res", C.c_int),
                ("grid_scale", C.c_float), ("grid_smoothstep", C.c_int), ("sh_degree", C.c_int),
                ("oneblob_bins", C.c_int), ("width", C.c_int), ("n_hidden", C.c_int), ("n_out", C.c_int),
                ("n_input", C.c_int), ("n_enc", C.c_int), ("n_enc_padded", C.c_int),
                ("n_out_padded", C.c_int), ("n_mlp_params", C.c_long), ("n_grid_params", C.c_long),
                ("n_params", C.c_long), ("n_entries", C.c_long), ("grid_offset", C.c_uint32 * 33)]


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        P = C.c_void_p
        L.nmgo_num_threads.restype = C.c_int
        L.nmgo_mixture_sample.argtypes = [C.c_int, P, C.c_int, C.c_int, C.c_long, P, P, C.POINTER(Opts), P, P, P]
        L.nmgo_mixture_boundary_distance.argtypes = [P, C.c_int, C.c_int, C.c_long, P, P, C.POINTER(Opts), P]
        L.nmgo_mixture_pdf.argtypes = [C.c_int, P, C.c_int, C.c_int, C.c_long, P, P, C.POINTER(Opts), P]
        L.nmgo_mixture_loss_grad.argtypes = [C.c_int, C.c_int, P, C.c_int, C.c_int, C.c_long, P, C.c_int,
                                             C.c_float, C.POINTER(Opts), P, P]
        L.nmgo_mixture_loss_grad.restype = C.c_double
        L.nmgo_net_init.argtypes = [C.POINTER(Net)]
        L.nmgo_featurize.argtypes = [C.POINTER(Net), C.c_long, P, P, P, P, P, P]
        L.nmgo_network_forward.argtypes = [C.POINTER(Net), P, C.c_long, P, P, P]
        L.nmgo_network_backward.argtypes = [C.POINTER(Net), P, C.c_long, P, P, P, P]
        L.nmgo_network_forward_f32.argtypes = [C.POINTER(Net), P, C.c_long, P, P]
        L.nmgo_network_backward_f32.argtypes = [C.POINTER(Net), P, C.c_long, P, P, P]
        L.nmgo_grid_backward.argtypes = [C.POINTER(Net), C.c_long, P, P, P]
        L.nmgo_adam_ema.argtypes = [C.c_long, C.c_long, P, C.c_float, C.c_float, C.c_float, C.c_float,
                                    C.c_float, C.c_float, C.c_float, C.c_uint32, P, P, P, P, P]
        _lib = L
    return _lib


def num_threads():
    return lib().nmgo_num_threads()


def _p(a):
    return None if a is None else a.ctypes.data


def _f32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float32)


def mixture_sample(raw, K, u4, cos_normal=None, fp64=True, o=None):
    raw, u4, cos_normal = _f32(raw), _f32(u4), _f32(cos_normal)
    n = raw.shape[0]
    d = np.zeros((n, 3), np.float64)
    p = np.zeros(n, np.float64)
    lb = np.zeros(n, np.int32)
    o = o or opts()
    lib().nmgo_mixture_sample(int(fp64), _p(raw), raw.shape[1], K, n, _p(u4), _p(cos_normal), C.byref(o),
                              _p(d), _p(p), _p(lb))
    return d, p, lb


def boundary_distance(raw, K, u4, cos_normal=None, o=None):
    raw, u4, cos_normal = _f32(raw), _f32(u4), _f32(cos_normal)
    n = raw.shape[0]
    out = np.zeros(n, np.float64)
    o = o or opts()
    lib().nmgo_mixture_boundary_distance(_p(raw), raw.shape[1], K, n, _p(u4), _p(cos_normal), C.byref(o), _p(out))
    return out


def mixture_pdf(raw, K, wi, cos_normal=None, fp64=True, o=None):
    raw, wi, cos_normal = _f32(raw), _f32(wi), _f32(cos_normal)
    n = raw.shape[0]
    p = np.zeros(n, np.float64)
    o = o or opts()
    lib().nmgo_mixture_pdf(int(fp64), _p(raw), raw.shape[1], K, n, _p(wi), _p(cos_normal), C.byref(o), _p(p))
    return p


def mixture_loss_grad(raw, K, samples, loss_scale=128.0, selection=False, fp64=True, o=None):
    """Returns (grad [n x stride] float64, loss [n] float64, FP64 loss sum)."""
    raw, samples = _f32(raw), _f32(samples)
    n = raw.shape[0]
    g = np.zeros(raw.shape, np.float64)
    loss = np.zeros(n, np.float64)
    o = o or opts()
    tot = lib().nmgo_mixture_loss_grad(int(fp64), int(selection), _p(raw), raw.shape[1], K, n, _p(samples),
                                       samples.shape[1], float(loss_scale), C.byref(o), _p(g), _p(loss))
    return g, loss, tot


def make_net(**kw):
    net = Net()
    for k, v in kw.items():
        setattr(net, k, v)
    lib().nmgo_net_init(C.byref(net))
    return net


def featurize(net, pos, wo, nrm, rough, aabb):
    pos, wo, nrm, rough, aabb = (_f32(x) for x in (pos, wo, nrm, rough, aabb))
    n = pos.shape[0]
    out = np.zeros((n, net.n_input), np.float32)
    lib().nmgo_featurize(C.byref(net), n, _p(pos), _p(wo), _p(nrm), _p(rough), _p(aabb), _p(out))
    return out


def network_forward(net, params, inputs, want_enc=False):
    params, inputs = _f32(params), _f32(inputs)
    n = inputs.shape[0]
    raw = np.zeros((n, net.n_out_padded), np.float64)
    enc = np.zeros((n, net.n_enc_padded), np.float64) if want_enc else None
    lib().nmgo_network_forward(C.byref(net), _p(params), n, _p(inputs), _p(raw), _p(enc))
    return (raw, enc) if want_enc else raw


def network_forward_f32(net, params, inputs):
    """The network forward in FP32 arithmetic (the CPU baseline's restatement; FP64 is the oracle)."""
    params, inputs = _f32(params), _f32(inputs)
    n = inputs.shape[0]
    raw = np.zeros((n, net.n_out_padded), np.float32)
    lib().nmgo_network_forward_f32(C.byref(net), _p(params), n, _p(inputs), _p(raw))
    return raw


def network_backward_f32(net, params, inputs, draw):
    """dL/dparams of the network in FP32 arithmetic (the CPU baseline's restatement)."""
    params, inputs, draw = _f32(params), _f32(inputs), _f32(draw)
    n = inputs.shape[0]
    dparams = np.zeros(net.n_params, np.float32)
    lib().nmgo_network_backward_f32(C.byref(net), _p(params), n, _p(inputs), _p(draw), _p(dparams))
    return dparams


def network_backward(net, params, inputs, draw, want_denc=False):
    params, inputs = _f32(params), _f32(inputs)
    draw = np.ascontiguousarray(draw, np.float64)
    n = inputs.shape[0]
    dparams = np.zeros(net.n_params, np.float64)
    denc = np.zeros((n, net.n_enc_padded), np.float64) if want_denc else None
    lib().nmgo_network_backward(C.byref(net), _p(params), n, _p(inputs), _p(draw), _p(dparams), _p(denc))
    return (dparams, denc) if want_denc else dparams


def grid_backward(net, inputs, denc):
    """Table gradient (FP64) from dL/d(encoded input) rows."""
    inputs = _f32(inputs)
    denc = np.ascontiguousarray(denc, np.float64)
    out = np.zeros(net.n_grid_params, np.float64)
    lib().nmgo_grid_backward(C.byref(net), inputs.shape[0], _p(inputs), _p(denc), _p(out))
    return out


def adam_ema(grad, loss_scale, lr, beta1, beta2, eps, l2, ema_decay, step, w, m, v, psteps, ema, n_matrix):
    """In-place Adam + EMA on float32 numpy arrays (psteps uint32)."""
    grad = _f32(grad)
    lib().nmgo_adam_ema(w.size, n_matrix, _p(grad), loss_scale, lr, beta1, beta2, eps, l2, ema_decay, step,
                        _p(w), _p(m), _p(v), _p(psteps), _p(ema))


# ------------------------------------------------------------ reference shim
def ref_lib():
    """The reference's own mixture code (None where it cannot be built)."""
    global _ref
    if _ref is None:
        path = build_oracle.build_reference()
        if path is None:
            return None
        L = C.CDLL(path)
        P = C.c_void_p
        L.ref_mixture_sample.argtypes = [P, C.c_int, C.c_long, P, P, P, P, P]
        L.ref_mixture_pdf.argtypes = [P, C.c_int, C.c_long, P, P, P]
        L.ref_dL_doutput_divergence.argtypes = [P, C.c_int, C.c_long, P, C.c_float, P, P]
        L.ref_generate_training_data.argtypes = [P] * 12 + [P, C.c_int, C.c_int] + [P] * 5 + [C.c_int, P, P]
        L.ref_generate_training_data.restype = C.c_int
        L.ref_generate_inference_data.argtypes = [P, P, P, P, C.c_int, P, P, P, P, P, P]
        L.ref_generate_inference_data.restype = C.c_int
        U = C.c_uint32
        L.ref_tcnn_grid_forward.argtypes = [C.c_int, C.c_int, P, U, C.c_float, C.c_int, C.c_int, P, P, U, P]
        L.ref_tcnn_grid_backward.argtypes = [C.c_int, C.c_int, P, U, C.c_float, C.c_int, C.c_int, P, U, P, P]
        L.ref_tcnn_grid_layout.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, C.c_int, C.c_int, P, P]
        L.ref_tcnn_snapshot_msgpack.argtypes = [P, C.c_uint64, C.c_int, P, C.c_long]
        L.ref_tcnn_snapshot_msgpack.restype = C.c_long
        L.ref_tcnn_sh.argtypes = [U, P, U, P]
        L.ref_tcnn_oneblob.argtypes = [U, P, U, U, P]
        L.ref_tcnn_adam_ema.argtypes = [U, U, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                                        C.c_float, U, C.c_int, P, P, P, P, P, P, P, P]
        _ref = L
    return _ref


def ref_mixture_sample(raw, u4, cos_normal=None):
    raw, u4, cos_normal = _f32(raw), _f32(u4), _f32(cos_normal)
    n = raw.shape[0]
    d = np.zeros((n, 3), np.float32)
    p = np.zeros(n, np.float32)
    lb = np.zeros(n, np.int32)
    ref_lib().ref_mixture_sample(_p(raw), raw.shape[1], n, _p(u4), _p(cos_normal), _p(d), _p(p), _p(lb))
    return d, p, lb


def ref_mixture_pdf(raw, wi, cos_normal=None):
    raw, wi, cos_normal = _f32(raw), _f32(wi), _f32(cos_normal)
    n = raw.shape[0]
    p = np.zeros(n, np.float32)
    ref_lib().ref_mixture_pdf(_p(raw), raw.shape[1], n, _p(wi), _p(cos_normal), _p(p))
    return p


def ref_loss_grad(raw, samples, loss_scale=128.0):
    """The reference's compute_dL_doutput_divergence kernel (train.cu:69-124) run on the host: __half raw
    outputs and gradients, per-sample likelihood."""
    raw, samples = _f32(raw), _f32(samples)
    n = raw.shape[0]
    g = np.zeros(raw.shape, np.float32)
    loss = np.zeros(n, np.float32)
    ref_lib().ref_dL_doutput_divergence(_p(raw), raw.shape[1], n, _p(samples), float(loss_scale), _p(g), _p(loss))
    return g, loss


def ref_extract_records(rec, cur_depth, offset, stride, train_res, res, aabb, capacity=None):
    """The reference's generate_training_data kernel (train.cu:14-67) run on the host over a
    GuidedPixelStateBuffer built from the per-depth arrays of `rec` (as extract_records takes them; every
    depth of the reference's MAX_TRAIN_DEPTH = 8 must be present). Returns (x [n, 9], records [n, 6]) in
    the reference's push order."""
    D = len(rec["L"])
    npx = int(np.asarray(cur_depth).size)

    def stack(k, w, dt=np.float32):
        return np.ascontiguousarray(np.stack([np.asarray(rec[k][d], dt).reshape(npx, w) for d in range(D)]))

    arrs = [stack("L", 3), stack("thp", 3), stack("pos", 3), stack("dir", 2), stack("wi_pdf", 1),
            stack("bsdf_pdf", 1), stack("mis_weight", 1), stack("delta", 1, np.uint8), stack("bsdf_val", 3),
            stack("wo", 2), stack("normal", 2), stack("roughness", 1)]
    cur = np.ascontiguousarray(np.asarray(cur_depth, np.uint32))
    u = [np.ascontiguousarray(np.asarray(v, np.uint32)) for v in (offset, stride, train_res, res)]
    box = _f32(np.asarray(aabb, np.float32))
    cap = int(capacity if capacity is not None else npx * D)
    L = ref_lib()
    ni, no = 9, 6
    x = np.zeros((cap, ni), np.float32)
    out = np.zeros((cap, no), np.float32)
    n = L.ref_generate_training_data(*[_p(a) for a in arrs], _p(cur), npx, D, *[_p(a) for a in u], _p(box), cap,
                                     _p(x), _p(out))
    n = min(n, cap)
    return x[:n], out[:n]


def ref_featurize_queue(pos, wo, normal, rough, aabb):
    """The reference's generate_inference_data kernel (train.cu:174-191) run on the host over a
    ScatterRayQueue (its soac-generated SOA<ScatterRayWorkItem>) filled with the given shading data.
    Returns (x [n, 9], leaves) where leaves holds the queue's own field arrays sd.pos / sd.wo / sd.frame.N
    ([n, 3]) and sd.roughness ([n]) as the SOA stores them."""
    pos, wo, normal, rough = (_f32(np.asarray(a, np.float32)) for a in (pos, wo, normal, rough))
    n = pos.shape[0]
    box = _f32(np.asarray(aabb, np.float32))
    x = np.zeros((n, 9), np.float32)
    lv = {k: np.zeros((n, 3), np.float32) for k in ("pos", "wo", "normal")}
    lv["roughness"] = np.zeros(n, np.float32)
    ni = ref_lib().ref_generate_inference_data(_p(pos), _p(wo), _p(normal), _p(rough), n, _p(box), _p(x),
                                               _p(lv["pos"]), _p(lv["wo"]), _p(lv["normal"]), _p(lv["roughness"]))
    assert ni == 9
    return x, lv


def extract_records(rec, cur_depth, offset, stride, train_res, res, aabb, input_mode=0, product=True,
                    selection=False, return_vertex=False):
    """Training records from per-pixel radiance records, restating the
    reference's generate_training_data (src/render/guided/train.cu:14-67) with
    normalizeSpatialCoord (train.h:173-177) in FP32, one IEEE operation at a
    time in the reference's order (numpy float32 scalars round every step), so
    the kept-record set, the positions and the radiance values are exact.

    Filter (train.cu:57-62): a vertex is dropped when the normalised position,
    the stored direction, the warped outgoing direction (product sampling, the
    reference's default, train.cu:36-37), the pdf or the local radiance
    L / thp * misWeight has a NaN, or the pdf is zero. The radiance is tested
    BEFORE the bsdfVal product (train.cu:50-53 multiply only output.L), so a
    NaN bsdfVal keeps the record with a NaN radiance.

    rec: dict of per-depth arrays [depth][pixels(, c)]: L, thp, pos, bsdf_val
    (3 channels), dir, wo, normal (2 angles), wi_pdf, bsdf_pdf, mis_weight,
    roughness, delta. Returns (x [n, 9|10], records [n, 6|7]) as float32 in
    the reference's loop order (training pixel, then depth); with
    return_vertex also the (pixel, depth) of every row [n, 2]."""
    f = np.float32
    aabb = np.asarray(aabb, np.float32)
    mn, mx = aabb[:3], aabb[3:]
    dg = mx - mn
    # AABB::inflate(diagonal().norm() * 0.005f): Eigen's unrolled sum is x^2 + (y^2 + z^2)
    infl = f(np.sqrt(f(dg[0] * dg[0]) + f(f(dg[1] * dg[1]) + f(dg[2] * dg[2])))) * f(0.005)
    lo, hi = mn - infl, mx + infl
    ctr = (lo + hi) / f(2)
    diag = hi - lo
    eps = f(1e-5)  # M_EPSILON (krrmath constants.h:25)
    xs, outs, verts = [], [], []
    with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
        for ty in range(train_res[1]):
            for tx in range(train_res[0]):
                px, py = tx * stride[0] + offset[0], ty * stride[1] + offset[1]
                if px >= res[0] or py >= res[1]:
                    continue
                pid = px + py * res[0]
                for d in range(min(int(cur_depth[pid]), len(rec["L"]))):
                    if rec["delta"][d][pid]:
                        continue
                    pos = rec["pos"][d][pid].astype(np.float32)
                    p = f(0.5) + (pos - ctr) / diag
                    th, ph = (f(v) for v in rec["wo"][d][pid])
                    wo = np.array([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], np.float32)
                    wdir = (wo + f(1)) * f(0.5)
                    nt, npf = (f(v) for v in rec["normal"][d][pid])
                    r = f(rec["roughness"][d][pid])
                    if input_mode == 0:
                        aux = [nt * f(1 / np.pi), npf * f(1 / (2 * np.pi)), f(1) - np.exp(-r)]
                    else:
                        n3 = np.array([np.sin(nt) * np.cos(npf), np.sin(nt) * np.sin(npf), np.cos(nt)], np.float32)
                        aux = list((n3 + f(1)) * f(0.5)) + [f(1) - np.exp(-r)]
                    thp = rec["thp"][d][pid].astype(np.float32)
                    Lr = rec["L"][d][pid].astype(np.float32)
                    L = np.array([Lr[c] / thp[c] if thp[c] > eps else f(0) for c in range(3)], np.float32)
                    L = L * f(rec["mis_weight"][d][pid])
                    Lout = L * rec["bsdf_val"][d][pid].astype(np.float32) if product else L
                    direc = rec["dir"][d][pid].astype(np.float32)
                    wi_pdf = f(rec["wi_pdf"][d][pid])
                    if (np.isnan(p).any() or np.isnan(direc).any() or np.isnan(wdir).any() or np.isnan(wi_pdf)
                            or wi_pdf == 0 or np.isnan(L).any()):
                        continue
                    xs.append(np.concatenate([p, wdir, np.array(aux, np.float32)]))
                    o = [direc[0], direc[1], Lout[0], Lout[1], Lout[2], wi_pdf]
                    if selection:
                        o.append(f(rec["bsdf_pdf"][d][pid]))
                    outs.append(o)
                    verts.append((pid, d))
    ni = 9 if input_mode == 0 else 10
    x = np.array(xs, np.float32).reshape(-1, ni)
    out = np.array(outs, np.float32).reshape(-1, 7 if selection else 6)
    if return_vertex:
        return x, out, np.array(verts, np.int64).reshape(-1, 2)
    return x, out


# ---------------------------------------------------------------------------
# tiny-cuda-nn 1.7's own kernels run on the host (oracle/ref_tcnn_kernels.cu):
# golden vectors for the encodings and the optimiser.
# ---------------------------------------------------------------------------
def ref_tcnn_grid_forward(feats, offsets, base_res, per_level_scale, hash_, smoothstep, table, pos):
    """kernel_grid (grid.h:220-384): features [n, levels * feats] of positions [n, 3] for a float table
    [offsets[-1] * feats]."""
    offsets = np.ascontiguousarray(offsets, np.uint32)
    levels = len(offsets) - 1
    pos, table = _f32(pos), _f32(table)
    n = pos.shape[0]
    enc = np.zeros((levels * feats, n), np.float32)
    r = ref_lib().ref_tcnn_grid_forward(feats, levels, _p(offsets), base_res, per_level_scale, int(hash_),
                                        int(smoothstep), _p(table), _p(pos), n, _p(enc))
    assert r == 0
    return np.ascontiguousarray(enc.T)


def ref_tcnn_grid_backward(feats, offsets, base_res, per_level_scale, hash_, smoothstep, pos, dl_dy):
    """kernel_grid_backward (grid.h:386-510): table gradient [offsets[-1] * feats] of dL/dfeatures
    dl_dy [n, levels * feats] at positions [n, 3] (FP32 accumulation, as tcnn's float gradient path)."""
    offsets = np.ascontiguousarray(offsets, np.uint32)
    levels = len(offsets) - 1
    pos = _f32(pos)
    n = pos.shape[0]
    dl = np.ascontiguousarray(np.asarray(dl_dy, np.float32).T)
    grad = np.zeros(int(offsets[-1]) * feats, np.float32)
    r = ref_lib().ref_tcnn_grid_backward(feats, levels, _p(offsets), base_res, per_level_scale, int(hash_),
                                         int(smoothstep), _p(pos), n, _p(dl), _p(grad))
    assert r == 0
    return grad


def ref_tcnn_sh(degree, x01):
    """kernel_sh (spherical_harmonics.h:126-153) of rows (d + 1) / 2: [n, degree^2]."""
    x01 = _f32(x01)
    n = x01.shape[0]
    out = np.zeros((n, degree * degree), np.float32)
    ref_lib().ref_tcnn_sh(degree, _p(x01), n, _p(out))
    return out


def ref_tcnn_oneblob(bins, vals):
    """kernel_one_blob_soa (oneblob.h:98-127): vals [n, dims] -> [n, dims * bins] (dimension-major)."""
    vals = _f32(vals)
    n, dims = vals.shape
    out = np.zeros((dims * bins, n), np.float32)
    ref_lib().ref_tcnn_oneblob(int(bins).bit_length() - 1, _p(vals), n, dims, _p(out))
    return np.ascontiguousarray(out.T)


def ref_tcnn_adam_ema(state, grad16, n_matrix, step, loss_scale=128.0, lr=1e-2, beta1=0.9, beta2=0.99, eps=1e-15,
                      l2_reg=1e-6, ema_decay=0.95, full_precision=True):
    """One EMA(Adam) step of tcnn (adam.h:47-119, ema.h:44-76) on `state` (dict of float32 arrays w_full, w16,
    m, v, ema16, ema_tmp and uint32 psteps, updated in place); grad16 holds the __half gradients as float."""
    n = state["w_full"].size
    grad16 = _f32(grad16)
    ref_lib().ref_tcnn_adam_ema(n, n_matrix, loss_scale, lr, beta1, beta2, eps, l2_reg, ema_decay, step,
                                int(full_precision), _p(state["w_full"]), _p(state["w16"]), _p(grad16),
                                _p(state["m"]), _p(state["v"]), _p(state["psteps"]), _p(state["ema16"]),
                                _p(state["ema_tmp"]))
    return state


def ref_tcnn_grid_layout(feats, levels, log2_hashmap, base_res, per_level_scale, hash_, smoothstep):
    """tcnn's GridEncodingTemplated constructor (grid.h:939-1000): the entry offset of every level
    [levels + 1] and the parameter count."""
    offsets = np.zeros(levels + 1, np.uint32)
    n_params = np.zeros(1, np.uint64)
    r = ref_lib().ref_tcnn_grid_layout(feats, levels, log2_hashmap, base_res, per_level_scale, int(hash_),
                                       int(smoothstep), _p(offsets), _p(n_params))
    assert r == 0
    return offsets, int(n_params[0])


def ref_tcnn_snapshot(params, params_type="__half"):
    """The bytes of a tcnn Trainer snapshot (Trainer::serialize, trainer.h:267-278, encoded by the reference's
    nlohmann::json::to_msgpack) holding `params` as __half or float."""
    p = np.ascontiguousarray(params, np.float16 if params_type == "__half" else np.float32)
    cap = p.nbytes + 256
    out = np.zeros(cap, np.uint8)
    n = ref_lib().ref_tcnn_snapshot_msgpack(_p(p), p.size, 0 if params_type == "__half" else 1, _p(out), cap)
    assert n > 0
    return out[:n].tobytes()
