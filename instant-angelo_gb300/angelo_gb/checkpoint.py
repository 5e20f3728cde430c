"""Checkpoint interop with the reference: its Lightning checkpoints load into
NeuSModel, and NeuSModel's state exports in the reference's form.

The reference restores weights with ``NeuSSystem.load_from_checkpoint(path,
strict=False)`` (launch.py:67, systems/__init__.py:11-15); the checkpoint's
``state_dict`` holds the system's tensors, the model's under ``model.``.
Module and parameter names line up one to one (tcnn's flat ``params`` of the
hash grid at ``geometry.encoding.encoding.encoding.params``, the
weight-normalised ``weight_g`` / ``weight_v`` of VanillaMLP layers, the
variance, ``scene_aabb``) except the occupancy grids, whose reference form is
nerfacc 0.3.3's OccupancyGrid buffers: ``_roi_aabb`` (6,), ``_binary`` (res,
res, res) bool, ``resolution`` (3,) int32, ``occs`` (res^3,), ``grid_coords``
(res^3, 3) and ``grid_indices`` (res^3,).  Here the grid keeps
``roi_aabb``, ``occs`` (same cell order, x-major) and the 1-bit mask ``bits``
(bit c % 32 of word c / 32).  nerfacc is not vendored with the reference: the
buffer names and shapes above restate its published 0.3.3 source."""
from __future__ import annotations

import torch

OCCUPANCY_PREFIXES = ("occupancy_grid.", "occupancy_grid_bg.")
_NERFACC_EXTRA = ("resolution", "grid_coords", "grid_indices")


def pack_bits(mask):
    """bool (N,) -> int32 words, bit c % 32 of word c // 32."""
    m = mask.reshape(-1).to(torch.int64)
    n = m.numel()
    pad = (-n) % 32
    if pad:
        m = torch.cat([m, m.new_zeros(pad)])
    w = (m.view(-1, 32) << torch.arange(32, device=m.device)).sum(-1)
    w = torch.where(w >= 2 ** 31, w - 2 ** 32, w)
    return w.to(torch.int32)


def unpack_bits(bits, n):
    b = bits.view(-1, 1).to(torch.int64) >> torch.arange(32, device=bits.device)
    return (b & 1).reshape(-1)[:n].to(torch.bool)


def from_reference(sd):
    """A reference checkpoint (or its ``state_dict``) -> a NeuSModel state_dict."""
    if "state_dict" in sd:
        sd = sd["state_dict"]
    out = {k[len("model."):]: v for k, v in sd.items() if k.startswith("model.")}
    for p in OCCUPANCY_PREFIXES:
        if p + "_binary" not in out:
            continue
        binary = out.pop(p + "_binary")
        out[p + "bits"] = pack_bits(binary.reshape(-1).to(torch.bool))
        out[p + "roi_aabb"] = out.pop(p + "_roi_aabb").float()
        for extra in _NERFACC_EXTRA:
            out.pop(p + extra, None)
    for k, v in out.items():
        if v.is_floating_point() and v.dtype != torch.float32:
            out[k] = v.float()
    return out


def to_reference(model):
    """NeuSModel -> the reference checkpoint's ``state_dict`` (keys under
    ``model.``; occupancy grids in nerfacc 0.3.3's form)."""
    sd = {k: v.detach().cpu() for k, v in model.state_dict().items()}
    out = {}
    for p in OCCUPANCY_PREFIXES:
        if p + "bits" not in sd:
            continue
        occs = sd.pop(p + "occs")
        res = round(occs.numel() ** (1.0 / 3.0))
        bits = sd.pop(p + "bits")
        out["model." + p + "_roi_aabb"] = sd.pop(p + "roi_aabb")
        out["model." + p + "_binary"] = unpack_bits(bits, occs.numel()).view(res, res, res)
        out["model." + p + "resolution"] = torch.tensor([res, res, res], dtype=torch.int32)
        out["model." + p + "occs"] = occs
        ax = torch.arange(res)
        out["model." + p + "grid_coords"] = torch.stack(
            torch.meshgrid(ax, ax, ax, indexing="ij"), -1).reshape(-1, 3)
        out["model." + p + "grid_indices"] = torch.arange(res ** 3)
    out.update({"model." + k: v for k, v in sd.items()})
    return out


def load_reference_checkpoint(model, ckpt, strict=True, trusted=False):
    """Load a reference checkpoint (a path or an already loaded dict) into
    ``model``; returns load_state_dict's (missing, unexpected) keys.

    A path is read with torch.load(weights_only=True): tensors and plain
    containers only.  A Lightning checkpoint that also pickles objects (its
    hyper-parameters) needs trusted=True, which unpickles everything in it:
    pass it only for files from a source you trust."""
    if isinstance(ckpt, (str, bytes)) or hasattr(ckpt, "__fspath__"):
        try:
            ckpt = torch.load(ckpt, map_location="cpu", weights_only=True)
        except Exception as e:   # noqa: BLE001 - the unpickler's refusal
            if not trusted:
                raise RuntimeError(
                    f"{ckpt}: holds objects other than tensors ({type(e).__name__}); "
                    "pass trusted=True to unpickle a checkpoint from a trusted source") from e
            ckpt = torch.load(ckpt, map_location="cpu", weights_only=False)
    return model.load_state_dict(from_reference(ckpt), strict=strict)
