"""sde_mc_gb300 — GB300-native Monte Carlo path integration with sde_mc's API.

Import surface mirrors sde_mc/__init__.py: every public name of the model,
solver, payoff, estimator and helper modules is re-exported here.
"""
from .version import __version__
from .sde import *
from .levy import *
from .options import *
from .helpers import *
from .schemes import *
from .solvers import *
from .mc import *
from .mlmc import *
from .nets import *
from .varred import *
from .problem import *
from . import torch_ops  # registers torch.ops.sdemc.*
