"""GB300-native neural parametric mixture guiding step -- Python host binding.

Thin ctypes layer over the C ABI of libnmg.so (declared in include/nmg.h).
Tensors are torch CUDA tensors; only their device pointers cross the ABI.
There is no CPU fallback: if the library is missing or was not built, every
call raises.

Mirrors the reference's guiding interface (src/render/guided/):
  mixture_sample / mixture_pdf / mixture_loss_grad -- MixedSphericalGaussian-
    Distribution's sample, pdf and the KL gradient kernel (distribution.h,
    train.cu:69-172), on raw network outputs;
  GuidingField -- the network-backed guide (GuidedPathTracer's inference and
    training steps, integrator.cpp:627-701).
"""
import ctypes as C
import os

from . import build as _build

_lib = None


class NMGError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("nmg status %d: %s" % (status, msg))
        self.status = status


class MixtureOpts(C.Structure):
    _fields_ = [("n_lobes", C.c_int), ("stride", C.c_int), ("kappa_softplus", C.c_int),
                ("kappa_poly", C.c_int), ("selection", C.c_int)]


def library_path():
    return _build.LIB


def lib():
    """Load libnmg.so (building it first if its sources are newer)."""
    global _lib
    if _lib is None:
        if os.environ.get("NMG_NO_BUILD") != "1":
            _build.build()
        if not os.path.exists(_build.LIB):
            raise NMGError(-1, "libnmg.so not built at %s" % _build.LIB)
        L = C.CDLL(_build.LIB)
        P = C.c_void_p
        L.nmg_status_string.restype = C.c_char_p
        L.nmg_status_string.argtypes = [C.c_int]
        L.nmg_last_error.restype = C.c_char_p
        L.nmg_version.restype = C.c_int
        L.nmg_mixture_sample.argtypes = [C.POINTER(MixtureOpts), P, P, P, C.c_int, P, P, P, P]
        L.nmg_mixture_pdf.argtypes = [C.POINTER(MixtureOpts), P, P, P, C.c_int, P, P]
        L.nmg_mixture_loss_workspace_bytes.restype = C.c_size_t
        L.nmg_mixture_loss_workspace_bytes.argtypes = [C.c_int]
        L.nmg_mixture_loss_grad.argtypes = [C.POINTER(MixtureOpts), P, P, C.c_int, C.c_int, C.c_float, P, P, P, P,
                                            C.c_size_t, P]
        for name in ("nmg_mixture_sample", "nmg_mixture_pdf", "nmg_mixture_loss_grad"):
            getattr(L, name).restype = C.c_int
        _lib = L
    return _lib


def check(status):
    if status != 0:
        L = lib()
        raise NMGError(status, "%s (%s)" % (L.nmg_status_string(status).decode(), L.nmg_last_error().decode()))


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream(stream):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def mixture_opts(n_lobes, stride, kappa_softplus=False, kappa_poly=True, selection=False):
    return MixtureOpts(n_lobes, stride, int(kappa_softplus), int(kappa_poly), int(selection))


def mixture_sample(raw, u4, n_lobes, cos_normal=None, kappa_softplus=False, want_lobe=True, stream=None):
    """Sample one direction per query: returns (dir [n,3], pdf [n], lobe [n] or None)."""
    import torch
    n = raw.shape[0]
    dev = raw.device
    d = torch.empty((n, 3), device=dev, dtype=torch.float32)
    p = torch.empty(n, device=dev, dtype=torch.float32)
    lb = torch.empty(n, device=dev, dtype=torch.int32) if want_lobe else None
    o = mixture_opts(n_lobes, raw.shape[1], kappa_softplus)
    check(lib().nmg_mixture_sample(C.byref(o), _ptr(raw), _ptr(u4), _ptr(cos_normal), n, _ptr(d), _ptr(p), _ptr(lb),
                                   _stream(stream)))
    return d, p, lb


def mixture_pdf(raw, wi, n_lobes, cos_normal=None, kappa_softplus=False, stream=None):
    import torch
    n = raw.shape[0]
    p = torch.empty(n, device=raw.device, dtype=torch.float32)
    o = mixture_opts(n_lobes, raw.shape[1], kappa_softplus)
    check(lib().nmg_mixture_pdf(C.byref(o), _ptr(raw), _ptr(wi), _ptr(cos_normal), n, _ptr(p), _stream(stream)))
    return p


def mixture_loss_grad(raw, records, n_lobes, loss_scale=128.0, selection=False, kappa_softplus=False,
                      kappa_poly=True, want_loss=True, stream=None):
    """KL loss gradient w.r.t. raw outputs: returns (grad [n,stride], loss [n] or None, loss_sum [1] float64)."""
    import torch
    n = raw.shape[0]
    dev = raw.device
    g = torch.zeros_like(raw)
    loss = torch.empty(n, device=dev, dtype=torch.float32) if want_loss else None
    tot = torch.empty(1, device=dev, dtype=torch.float64)
    L = lib()
    wsb = L.nmg_mixture_loss_workspace_bytes(n)
    ws = torch.empty(wsb, device=dev, dtype=torch.uint8)
    o = mixture_opts(n_lobes, raw.shape[1], kappa_softplus, kappa_poly, selection)
    check(L.nmg_mixture_loss_grad(C.byref(o), _ptr(raw), _ptr(records), records.shape[1], n, float(loss_scale),
                                  _ptr(g), _ptr(loss), _ptr(tot), _ptr(ws), wsb, _stream(stream)))
    return g, loss, tot


# ---------------------------------------------------------------- guiding field
PRESET_REFERENCE = 0
PRESET_HASHGRID = 1
PATH_FP32, PATH_BF16, PATH_FP16 = 0, 1, 2


class Config(C.Structure):
    _fields_ = [("n_lobes", C.c_int), ("selection", C.c_int), ("kappa_softplus", C.c_int), ("kappa_poly", C.c_int),
                ("cosine_aware", C.c_int), ("input_mode", C.c_int), ("grid_hash", C.c_int),
                ("grid_levels", C.c_int), ("grid_features", C.c_int), ("grid_log2_hashmap", C.c_int),
                ("grid_base_resolution", C.c_int), ("grid_per_level_scale", C.c_float),
                ("grid_smoothstep", C.c_int), ("sh_degree", C.c_int), ("oneblob_bins", C.c_int),
                ("aabb", C.c_float * 6), ("width", C.c_int), ("hidden_layers", C.c_int), ("path", C.c_int),
                ("learning_rate", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float), ("epsilon", C.c_float),
                ("l2_reg", C.c_float), ("ema_decay", C.c_float), ("use_ema", C.c_int), ("loss_scale", C.c_float),
                ("seed", C.c_uint32)]


class Info(C.Structure):
    _fields_ = [("n_input", C.c_int), ("n_encoded", C.c_int), ("n_encoded_padded", C.c_int), ("n_output", C.c_int),
                ("n_output_padded", C.c_int), ("n_mlp_params", C.c_int64), ("n_grid_params", C.c_int64),
                ("n_params", C.c_int64), ("grid_entries", C.c_int64), ("record_floats", C.c_int)]


class Shading(C.Structure):
    _fields_ = [("pos", C.c_void_p), ("wo", C.c_void_p), ("normal", C.c_void_p), ("roughness", C.c_void_p)]


class QueryOut(C.Structure):
    _fields_ = [("dir", C.c_void_p), ("pdf", C.c_void_p), ("lobe", C.c_void_p), ("raw", C.c_void_p),
                ("selection", C.c_void_p)]


class Bounce(C.Structure):
    _fields_ = [("in_", Shading), ("u4", C.c_void_p), ("d_count", C.c_void_p), ("n_max", C.c_int),
                ("out", QueryOut), ("train_x", C.c_void_p), ("train_records", C.c_void_p),
                ("train_count", C.c_void_p), ("train_n_max", C.c_int), ("stats", C.c_void_p)]


class RecordArrays(C.Structure):
    _fields_ = [(name, C.c_void_p) for name in ("L", "thp", "pos", "dir", "wi_pdf", "bsdf_pdf", "mis_weight", "delta",
                                               "bsdf_val", "wo", "normal", "roughness")]


MAX_TRAIN_DEPTH = 8


class RadianceRecords(C.Structure):
    _fields_ = [("max_depth", C.c_int), ("product", C.c_int), ("cur_depth", C.c_void_p),
                ("depth", RecordArrays * MAX_TRAIN_DEPTH)]


class TrainPixels(C.Structure):
    _fields_ = [("offset", C.c_uint * 2), ("stride", C.c_uint * 2), ("train_res", C.c_uint * 2), ("res", C.c_uint * 2)]


def _bind_field(L):
    P = C.c_void_p
    sig = {
        "nmg_config_init": [C.POINTER(Config), C.c_int],
        "nmg_config_info": [C.POINTER(Config), C.POINTER(Info)],
        "nmg_create": [C.POINTER(Config), C.POINTER(P)],
        "nmg_get_info": [P, C.POINTER(Info)],
        "nmg_reserve": [P, C.c_int, C.c_int],
        "nmg_device_bytes": [P, C.POINTER(C.c_uint64)],
        "nmg_set_params": [P, P, P],
        "nmg_get_params": [P, C.c_int, P, P],
        "nmg_get_gradients": [P, P, P],
        "nmg_featurize": [P, C.POINTER(Shading), C.c_int, P, P],
        "nmg_infer_raw": [P, P, C.c_int, C.c_int, P, P],
        "nmg_query": [P, C.POINTER(Shading), P, P, C.c_int, C.POINTER(QueryOut), P],
        "nmg_pdf": [P, C.POINTER(Shading), P, P, C.c_int, P, P],
        "nmg_train_step": [P, P, P, P, C.c_int, P, P],
        "nmg_query_host": [P, C.POINTER(Shading), P, C.c_int, C.POINTER(QueryOut), P],
        "nmg_train_step_host": [P, P, P, C.c_int, P, P],
        "nmg_frame_capture": [P, C.POINTER(Bounce), C.c_int, C.POINTER(P)],
        "nmg_frame_launch": [P, P],
        "nmg_frame_run_eager": [P, C.POINTER(Bounce), C.c_int, P],
        "nmg_network_vjp": [P, P, P, C.c_int, P, P, P],
        "nmg_set_query_tiling": [P, C.c_int],
        "nmg_set_host_chunks": [P, C.c_int],
        "nmg_autotune_query": [P, C.POINTER(Shading), P, C.c_int, C.POINTER(QueryOut), C.c_int, C.POINTER(C.c_int), P],
        "nmg_check_errors": [P],
        "nmg_selftest_wait_timeout": [P, P],
        "nmg_save": [P, C.c_char_p],
        "nmg_export_tcnn": [P, C.c_char_p, C.c_int],
        "nmg_extract_records": [P, C.POINTER(RadianceRecords), C.POINTER(TrainPixels), C.c_int, P, P, P, P],
        "nmg_train_frame": [P, C.POINTER(RadianceRecords), C.POINTER(TrainPixels), C.c_int, P, P, C.c_int, C.c_int,
                            C.c_int, P, P],
        "nmg_import_tcnn": [P, C.c_char_p, P],
        "nmg_load": [P, C.c_char_p],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
    L.nmg_destroy.argtypes = [P]
    L.nmg_destroy.restype = None
    L.nmg_get_step.argtypes = [P]
    L.nmg_get_step.restype = C.c_int
    L.nmg_get_query_tiling.argtypes = [P]
    L.nmg_get_query_tiling.restype = C.c_int
    L.nmg_get_host_chunks.argtypes = [P]
    L.nmg_get_host_chunks.restype = C.c_int
    L.nmg_frame_nodes.argtypes = [P]
    L.nmg_frame_nodes.restype = C.c_int
    L.nmg_frame_destroy.argtypes = [P]
    L.nmg_frame_destroy.restype = None


def config(preset=PRESET_HASHGRID, **overrides):
    cfg = Config()
    L = lib()
    if not hasattr(L, "_field_bound"):
        _bind_field(L)
        L._field_bound = True
    check(L.nmg_config_init(C.byref(cfg), preset))
    for k, v in overrides.items():
        if k == "aabb":
            for i in range(6):
                cfg.aabb[i] = float(v[i])
        else:
            setattr(cfg, k, v)
    return cfg


def config_info(cfg):
    """nmg_config_info: the sizes a configuration implies (no device needed)."""
    L = lib()
    if not hasattr(L, "_field_bound"):
        _bind_field(L)
        L._field_bound = True
    info = Info()
    check(L.nmg_config_info(C.byref(cfg), C.byref(info)))
    return info


class GuidingField:
    """The network-backed guiding distribution (encoding -> MLP -> vMF mixture).

    Mirrors GuidedPathTracer's guiding members (src/render/guided/
    integrator.cpp): `query` is inferenceStep + the guided sample/pdf,
    `pdf` the MIS pdf, `train_step` one batch of trainStep.
    """

    def __init__(self, cfg=None, max_queries=0, max_batch=0):
        self.L = lib()
        if not hasattr(self.L, "_field_bound"):
            _bind_field(self.L)
            self.L._field_bound = True
        self.cfg = cfg if cfg is not None else config()
        h = C.c_void_p()
        check(self.L.nmg_create(C.byref(self.cfg), C.byref(h)))
        self.h = h
        self.info = Info()
        check(self.L.nmg_get_info(self.h, C.byref(self.info)))
        if max_queries or max_batch:
            self.reserve(max_queries, max_batch)

    def close(self):
        if getattr(self, "h", None):
            self.L.nmg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def reserve(self, max_queries, max_batch):
        check(self.L.nmg_reserve(self.h, int(max_queries), int(max_batch)))

    @property
    def device_bytes(self):
        """Device memory the field holds (parameters, optimiser state, workspaces)."""
        b = C.c_uint64()
        check(self.L.nmg_device_bytes(self.h, C.byref(b)))
        return int(b.value)

    @property
    def n_params(self):
        return int(self.info.n_params)

    def get_params(self, which=0):
        import torch
        out = torch.empty(self.n_params, device="cuda", dtype=torch.float32)
        check(self.L.nmg_get_params(self.h, which, _ptr(out), _stream(None)))
        return out

    def set_params(self, params):
        check(self.L.nmg_set_params(self.h, _ptr(params), _stream(None)))

    def operand_params(self, which=1):
        """The parameter values the fused kernels multiply, as FP32 (None on the plain FP32 path):
        the grid table in the path's 16-bit format; the MLP of the training image (which = 0) all in
        that format; the MLP of the inference image (which = 1, the query and pdf passes) in FP16 on
        both 16-bit paths."""
        import torch
        if self.cfg.path == PATH_FP32:
            return None
        p = self.get_params(which)
        n_mlp = int(self.info.n_mlp_params)
        if self.cfg.path == PATH_FP16:
            return p.to(torch.float16).float()
        out = p.to(torch.bfloat16).float()
        if which == 1:
            out[:n_mlp] = p[:n_mlp].to(torch.float16).float()
        return out

    def get_gradients(self):
        import torch
        out = torch.empty(self.n_params, device="cuda", dtype=torch.float32)
        check(self.L.nmg_get_gradients(self.h, _ptr(out), _stream(None)))
        return out

    @property
    def step(self):
        return self.L.nmg_get_step(self.h)

    @staticmethod
    def shading(pos, wo, normal, rough):
        return Shading(pos.data_ptr(), wo.data_ptr(), normal.data_ptr(), rough.data_ptr())

    def featurize(self, pos, wo, normal, rough, stream=None):
        import torch
        n = pos.shape[0]
        x = torch.empty((n, self.info.n_input), device="cuda", dtype=torch.float32)
        sh = self.shading(pos, wo, normal, rough)
        check(self.L.nmg_featurize(self.h, C.byref(sh), n, _ptr(x), _stream(stream)))
        return x

    def infer_raw(self, x, which=1, stream=None):
        import torch
        n = x.shape[0]
        raw = torch.empty((n, self.info.n_output_padded), device="cuda", dtype=torch.float32)
        check(self.L.nmg_infer_raw(self.h, _ptr(x), n, which, _ptr(raw), _stream(stream)))
        return raw

    def query(self, pos, wo, normal, rough, u4, count=None, want_raw=False, outputs=None, stream=None):
        """Returns dict(dir, pdf, lobe, raw?, selection?) for the first count (device int tensor) queries."""
        import torch
        n = pos.shape[0]
        if outputs is None:
            outputs = {
                "dir": torch.empty((n, 3), device="cuda"),
                "pdf": torch.empty(n, device="cuda"),
                "lobe": torch.empty(n, device="cuda", dtype=torch.int32),
            }
            if want_raw:
                outputs["raw"] = torch.empty((n, self.info.n_output_padded), device="cuda")
            if self.cfg.selection:
                outputs["selection"] = torch.empty(n, device="cuda")
        o = QueryOut(*(outputs[k].data_ptr() if outputs.get(k) is not None else None
                       for k in ("dir", "pdf", "lobe", "raw", "selection")))
        sh = self.shading(pos, wo, normal, rough)
        check(self.L.nmg_query(self.h, C.byref(sh), _ptr(u4), _ptr(count), n, C.byref(o), _stream(stream)))
        return outputs

    def pdf(self, pos, wo, normal, rough, wi, count=None, stream=None):
        import torch
        n = pos.shape[0]
        p = torch.empty(n, device="cuda")
        sh = self.shading(pos, wo, normal, rough)
        check(self.L.nmg_pdf(self.h, C.byref(sh), _ptr(wi), _ptr(count), n, _ptr(p), _stream(stream)))
        return p

    def train_step(self, x, records, count=None, stats=None, stream=None):
        """One optimiser step; returns a float64 device tensor [mean loss, grad norm]."""
        import torch
        if stats is None:
            stats = torch.zeros(2, device="cuda", dtype=torch.float64)
        check(self.L.nmg_train_step(self.h, _ptr(x), _ptr(records), _ptr(count), x.shape[0], _ptr(stats),
                                    _stream(stream)))
        return stats

    def query_host(self, pos, wo, normal, rough, u4, outputs, stream=None):
        """nmg_query on host tensors (pinned for overlap); outputs: dict of host tensors dir, pdf[, lobe,
        selection]. Asynchronous on `stream`: synchronise before reading the outputs."""
        o = QueryOut(*(outputs[k].data_ptr() if outputs.get(k) is not None else None
                       for k in ("dir", "pdf", "lobe", "raw", "selection")))
        sh = self.shading(pos, wo, normal, rough)
        check(self.L.nmg_query_host(self.h, C.byref(sh), _ptr(u4), pos.shape[0], C.byref(o), _stream(stream)))
        return outputs

    def train_step_host(self, x, records, stats=None, stream=None):
        """nmg_train_step on host tensors; stats (host float64 [2], may be None) receives the statistics."""
        check(self.L.nmg_train_step_host(self.h, _ptr(x), _ptr(records), x.shape[0], _ptr(stats), _stream(stream)))
        return stats

    @staticmethod
    def bounce(pos, wo, normal, rough, u4, outputs, count=None, n_max=None, train=None):
        """One bounce of a frame: device tensors of the queue (capacity n_max = pos rows), its device
        count (int32 tensor or None), output tensors, and optionally a training batch
        train = (x, records, count or None, stats or None)."""
        b = Bounce()
        b.in_ = GuidingField.shading(pos, wo, normal, rough)
        b.u4 = u4.data_ptr()
        b.d_count = count.data_ptr() if count is not None else None
        b.n_max = int(n_max if n_max is not None else pos.shape[0])
        b.out = QueryOut(*(outputs[k].data_ptr() if outputs.get(k) is not None else None
                           for k in ("dir", "pdf", "lobe", "raw", "selection")))
        if train is not None:
            x, rec, cnt, st = train
            b.train_x, b.train_records = x.data_ptr(), rec.data_ptr()
            b.train_count = cnt.data_ptr() if cnt is not None else None
            b.train_n_max = int(x.shape[0])
            b.stats = st.data_ptr() if st is not None else None
        # the structure holds raw device pointers: keep the tensors (the count in particular,
        # which callers often create inline) alive for as long as the bounce is
        b._keep = (pos, wo, normal, rough, u4, dict(outputs), count, train)
        return b

    def capture_frame(self, bounces):
        """CUDA graph of the bounce loop (nmg_frame_capture); returns a Frame."""
        arr = (Bounce * len(bounces))(*bounces)
        h = C.c_void_p()
        check(self.L.nmg_frame_capture(self.h, arr, len(bounces), C.byref(h)))
        # the graph replays with the bounces' device pointers: the frame keeps their tensors alive
        return Frame(self.L, h, (arr, [getattr(b, "_keep", None) for b in bounces]))

    def run_frame_eager(self, bounces, stream=None):
        arr = (Bounce * len(bounces))(*bounces)
        check(self.L.nmg_frame_run_eager(self.h, arr, len(bounces), _stream(stream)))

    def vjp(self, x, draw, dparams=None, stream=None):
        import torch
        n = x.shape[0]
        raw = torch.empty((n, self.info.n_output_padded), device="cuda")
        if dparams is None:
            dparams = torch.zeros(self.n_params, device="cuda")
        check(self.L.nmg_network_vjp(self.h, _ptr(x), _ptr(draw), n, _ptr(raw), _ptr(dparams), _stream(stream)))
        return raw, dparams

    def set_query_tiling(self, warpgroups_per_cta):
        check(self.L.nmg_set_query_tiling(self.h, int(warpgroups_per_cta)))

    @property
    def query_tiling(self):
        return self.L.nmg_get_query_tiling(self.h)

    def set_host_chunks(self, chunks):
        """Most chunks query_host splits a wavefront into (0 = automatic)."""
        check(self.L.nmg_set_host_chunks(self.h, int(chunks)))

    @property
    def host_chunks(self):
        return self.L.nmg_get_host_chunks(self.h)

    def autotune(self, pos, wo, normal, rough, u4, use_cache=False, stream=None):
        """Picks the fastest fused-query tiling on these inputs; returns it."""
        import torch
        n = pos.shape[0]
        out = {"dir": torch.empty((n, 3), device="cuda"), "pdf": torch.empty(n, device="cuda")}
        o = QueryOut(out["dir"].data_ptr(), out["pdf"].data_ptr(), None, None, None)
        sh = self.shading(pos, wo, normal, rough)
        chosen = C.c_int(0)
        check(self.L.nmg_autotune_query(self.h, C.byref(sh), _ptr(u4), n, C.byref(o), int(use_cache),
                                        C.byref(chosen), _stream(stream)))
        return chosen.value

    def check_errors(self):
        check(self.L.nmg_check_errors(self.h))

    def selftest_wait_timeout(self, stream=None):
        """Runs a kernel whose bounded device wait gives up (about a second); the next
        check_errors() raises NMGError with NMG_ERR_TIMEOUT."""
        check(self.L.nmg_selftest_wait_timeout(self.h, _stream(stream)))

    @staticmethod
    def _records(records, cur_depth, offset, stride, train_res, res, product):
        r = RadianceRecords()
        r.max_depth = len(records)
        r.product = int(product)
        r.cur_depth = cur_depth.data_ptr()
        for d, arrays in enumerate(records):
            for name, _ in RecordArrays._fields_:
                t = arrays.get(name)
                setattr(r.depth[d], name, t.data_ptr() if t is not None else None)
        tp = TrainPixels((C.c_uint * 2)(*offset), (C.c_uint * 2)(*stride), (C.c_uint * 2)(*train_res),
                         (C.c_uint * 2)(*res))
        return r, tp

    def extract_records(self, records, cur_depth, offset, stride, train_res, res, capacity, product=True,
                        stream=None, outputs=None):
        """nmg_extract_records: records = list (one per depth) of dicts of device tensors (L, thp, pos, dir,
        wi_pdf, bsdf_pdf, mis_weight, delta (uint8), bsdf_val, wo, normal, roughness). Returns
        (x [capacity, n_input], records [capacity, record_floats], count (device int32 [1])); `outputs`
        = such a triple to write into instead."""
        import torch
        r, tp = self._records(records, cur_depth, offset, stride, train_res, res, product)
        if outputs is not None:
            x, rec, cnt = outputs  # nmg_extract_records resets the count itself
        else:
            x = torch.zeros((capacity, self.info.n_input), device="cuda")
            rec = torch.zeros((capacity, self.info.record_floats), device="cuda")
            cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
        check(self.L.nmg_extract_records(self.h, C.byref(r), C.byref(tp), int(capacity), _ptr(x), _ptr(rec),
                                         _ptr(cnt), _stream(stream)))
        return x, rec, cnt

    def train_frame(self, records, cur_depth, offset, stride, train_res, res, capacity, batch_size, max_batches,
                    min_batch, product=True, stream=None, outputs=None):
        """nmg_train_frame: one frame's training on its radiance records (arguments as extract_records).
        Returns (vertex ids (device int32 [capacity], the uint32 ids), count (device int32 [1]), stats
        (device float64 [max_batches, 2]))."""
        import torch
        r, tp = self._records(records, cur_depth, offset, stride, train_res, res, product)
        if outputs is not None:
            ids, cnt, stats = outputs
        else:
            ids = torch.zeros(max(int(capacity), 1), dtype=torch.int32, device="cuda")
            cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
            stats = torch.zeros((max_batches, 2), dtype=torch.float64, device="cuda")
        check(self.L.nmg_train_frame(self.h, C.byref(r), C.byref(tp), int(capacity), _ptr(ids), _ptr(cnt),
                                     int(batch_size), int(max_batches), int(min_batch), _ptr(stats),
                                     _stream(stream)))
        return ids, cnt, stats

    def export_tcnn(self, path, params_type="__half"):
        """Inference parameters as a tiny-cuda-nn Trainer snapshot (MessagePack)."""
        check(self.L.nmg_export_tcnn(self.h, str(path).encode(), {"__half": 0, "float": 1}[params_type]))

    def import_tcnn(self, path, stream=None):
        check(self.L.nmg_import_tcnn(self.h, str(path).encode(), _stream(stream)))

    def save(self, path):
        check(self.L.nmg_save(self.h, path.encode()))

    def load(self, path):
        check(self.L.nmg_load(self.h, path.encode()))


class Frame:
    """A captured bounce loop (CUDA graph executable)."""

    def __init__(self, L, h, bounces):
        self.L, self.h, self._bounces = L, h, bounces

    @property
    def nodes(self):
        return self.L.nmg_frame_nodes(self.h)

    def launch(self, stream=None):
        check(self.L.nmg_frame_launch(self.h, _stream(stream)))

    def close(self):
        if self.h:
            self.L.nmg_frame_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def oracle_net_spec(cfg):
    """Keyword arguments for the oracle's network description of a config."""
    return dict(input_mode=cfg.input_mode, grid_hash=cfg.grid_hash, grid_levels=cfg.grid_levels,
                grid_feats=cfg.grid_features, grid_log2_T=cfg.grid_log2_hashmap,
                grid_base_res=cfg.grid_base_resolution, grid_scale=cfg.grid_per_level_scale,
                grid_smoothstep=cfg.grid_smoothstep, sh_degree=cfg.sh_degree, oneblob_bins=cfg.oneblob_bins,
                width=cfg.width, n_hidden=cfg.hidden_layers, n_out=4 * cfg.n_lobes + (1 if cfg.selection else 0))
