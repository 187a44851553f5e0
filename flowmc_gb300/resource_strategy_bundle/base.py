"""ResourceStrategyBundle (mirrors resource_strategy_bundle/base.py:7-17)."""
from __future__ import annotations

from abc import ABC


class ResourceStrategyBundle(ABC):
    resources: dict
    strategies: dict
    strategy_order: list
