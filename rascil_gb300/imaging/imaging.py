"""Context dispatcher, as ``rascil/processing_components/imaging/imaging.py:26-93``.

Contexts served here: ``"ng"`` (w-stacking on), ``"2d"`` (the same without
w-stacking) and ``"gb"`` (alias of ``"ng"``).  The reference's
``"awprojection"`` and ``"wg"`` contexts are other algorithms and raise.
"""
from .ng import invert_ng, predict_ng


def predict_blockvisibility(vis, model, context="ng", gcfcf=None, **kwargs):
    if context == "2d":
        return predict_ng(vis, model, do_wstacking=False, **kwargs)
    if context in ("ng", "gb"):
        return predict_ng(vis, model, **kwargs)
    raise ValueError(f"Unknown imaging context {context}")


def invert_blockvisibility(vis, im, dopsf=False, normalise=True, context="ng", gcfcf=None,
                           **kwargs):
    if context == "2d":
        return invert_ng(vis, im, dopsf=dopsf, normalise=normalise, do_wstacking=False,
                         **kwargs)
    if context in ("ng", "gb"):
        return invert_ng(vis, im, dopsf=dopsf, normalise=normalise, **kwargs)
    raise ValueError(f"Unknown imaging context {context}")
