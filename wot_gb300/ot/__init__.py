"""wot.ot on the GPU: solvers, OTModel, configuration parsing, local PCA."""
from .initializer import (parse_configuration, parse_parameter_file, parse_per_timepair_configuration,
                          parse_per_timepoint_configuration)
from .optimal_transport import (compute_transport_matrix, dual, fdiv, fdivstar, optimal_transport_duality_gap,
                                primal, transport_stablev2)
from .ot_model import OTModel
from .util import compute_pca_reference_api as compute_pca  # the reference's return values
