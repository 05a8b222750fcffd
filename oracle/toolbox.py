"""Oracle: noise estimate, thresholding, source extraction, SNR.

Restates pymoresane/iuwt_toolbox.py:

* ``estimate_threshold`` -- :17-48. Per scale sigma = median(|w[mask]|)/0.6745,
  the mask excluding an edge band of width edge_excl and a central square of
  half-width int_excl around (mid, mid), mid = shape[1] // 2. The median of
  a float32 array is computed by numpy in float32 (mean of the two middle
  order statistics for even counts), then divided by 0.6745 in float32 and
  stored in a float64 array -- exactly what the reference computes on the
  float32 coefficients that its GPU path returns.
* ``apply_threshold``    -- :50-75, w * (|w| > sigma_level * sigma) (strict).
* ``source_extraction``  -- cpu_source_extraction :97-154 (``semantics='cpu'``,
  tolerance * max in float64) and gpu_source_extraction :156-290
  (``semantics='gpu'``, tolerance * max rounded to float32): 8-connected
  labels of w != 0 per scale (scipy.ndimage.label), islands kept top-down if
  any pixel satisfies w >= tol * max_s (|w| with neg_comp) and, below the top
  scale, lies inside the kept mask of the scale above. Returns
  (mask * w as float64, mask as int32).
* ``snr_ratio``          -- :292-306, 20 log10(||a|| / ||a - b||).
* ``label``              -- scipy.ndimage.label with the 3 x 3 structure
  (the reference's connectivity); labels numbered in raster order of each
  component's first pixel.
"""
import numpy as np
from scipy import ndimage

STRUCT8 = [[1, 1, 1], [1, 1, 1], [1, 1, 1]]


def noise_mask(shape, edge_excl=0, int_excl=0):
    """Boolean mask of the pixels used by the MAD estimate (iuwt_toolbox.py:26-43)."""
    ny, nx = shape
    mid = ny // 2 if False else shape[1] // 2  # the reference uses in1.shape[1]/2 for both axes
    if (edge_excl != 0) | (int_excl != 0):
        if edge_excl != 0:
            mask = np.zeros([ny, nx])
            mask[edge_excl:-edge_excl, edge_excl:-edge_excl] = 1
        else:
            mask = np.ones([ny, nx])
        if int_excl != 0:
            mask[mid - int_excl:mid + int_excl, mid - int_excl:mid + int_excl] = 0
    else:
        mask = np.ones([ny, nx])
    return mask == 1


def estimate_threshold(in1, edge_excl=0, int_excl=0):
    out = np.empty([in1.shape[0]])
    mask = noise_mask(in1.shape[1:], edge_excl, int_excl)
    for i in range(in1.shape[0]):
        out[i] = np.median(np.abs(in1[i, mask])) / 0.6745
    return out


def apply_threshold(in1, threshold, sigma_level=4):
    if in1.ndim == 2:
        return (np.abs(in1) > (sigma_level * threshold)) * in1
    out = np.empty_like(in1)
    for i in range(in1.shape[0]):
        out[i] = (np.abs(in1[i]) > (sigma_level * threshold[i])) * in1[i]
    return out


def label(mask):
    return ndimage.label(mask, structure=STRUCT8)


def source_extraction(in1, tolerance, neg_comp=False, semantics="gpu"):
    s = in1.shape[0]
    maxima = np.empty([s, 1], dtype=np.float32 if semantics == "gpu" else np.float64)
    objects = np.empty(in1.shape, dtype=np.int32)
    for i in range(s):
        maxima[i] = np.max(np.abs(in1[i])) if neg_comp else np.max(in1[i])
        objects[i], _ = label(in1[i])
    for i in range(s - 1, -1, -1):
        cond = tolerance * maxima[i]
        sig = (np.abs(in1[i]) >= cond) if neg_comp else (in1[i] >= cond)
        cand = sig * objects[i]
        if i < s - 1:
            cand = cand * objects[i + 1]
        keep = np.unique(cand[cand > 0])
        page = objects[i]
        kept = np.isin(page, keep) & (page > 0)
        objects[i] = kept.astype(np.int32)
    return objects * in1, objects


def snr_ratio(in1, in2):
    return 20 * (np.log10(np.linalg.norm(in1) / np.linalg.norm(in1 - in2)))
