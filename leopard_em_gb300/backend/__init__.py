"""Backend functions with Leopard-EM's signatures (leopard_em/backend/__init__.py)."""

from .core_match_template import MatchTemplateSearch, core_match_template

__all__ = ["core_match_template", "MatchTemplateSearch"]
