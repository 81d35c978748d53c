"""Imports the product package (its directory name is not a Python identifier)."""
import importlib
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NAME = "fine-grained-differentiable-physics-a-yarn-level-model-for-fabrics_gb300"
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
ys = importlib.import_module(NAME)


def spec_from_golden(g):
    import goldens
    return ys.ClothSpec(**goldens.spec_kwargs(g))


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
