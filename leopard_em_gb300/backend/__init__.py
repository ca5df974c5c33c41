"""Backend functions with Leopard-EM's signatures (leopard_em/backend/__init__.py)."""

from .core_match_template import MatchTemplateSearch, core_match_template
from .core_refine_template import core_refine_template, cross_correlate_particle_stack

__all__ = ["core_match_template", "core_refine_template", "cross_correlate_particle_stack", "MatchTemplateSearch"]
