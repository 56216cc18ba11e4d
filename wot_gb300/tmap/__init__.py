"""wot.tmap on the GPU: TransportMapModel, chaining and helpers."""
from .chaining import chain_transport_maps, find_path
from .transport_map_model import TransportMapModel
from .util import glue_transport_maps, unique_timepoint
