"""GB300-native (sm_103a) 2DTM search with Leopard-EM's backend API.

``leopard_em_gb300.backend.core_match_template`` is a drop-in for
``leopard_em.backend.core_match_template`` (same arguments, same returned
keys); the work runs in hand-written CUDA kernels loaded from the in-tree
library built by ``leopard_em_gb300.build``.
"""

__version__ = "0.1.0"
