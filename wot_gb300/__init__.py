"""GB300-native (sm_103a) implementation of Waddington-OT's transport-map path.

Drop-in for the corresponding parts of ``wot``:

* ``wot_gb300.ot``   — ``OTModel``, ``compute_transport_matrix``,
  ``optimal_transport_duality_gap``, ``transport_stablev2``, configuration parsing;
* ``wot_gb300.tmap`` — ``TransportMapModel`` (push-forward, pull-back, ancestors,
  descendants, fates, trajectories, transition tables, chaining);
* ``wot_gb300.Population``.

All compute runs in libwotg.so (hand-written CUDA, C ABI in include/wotg.h);
there is no CPU fallback.
"""
from . import ot, tmap
from .dataset import Dataset, Frame
from .ot import OTModel
from .population import Population
from .tmap import TransportMapModel

__all__ = ['ot', 'tmap', 'OTModel', 'TransportMapModel', 'Population', 'Dataset', 'Frame']
