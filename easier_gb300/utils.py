"""Logger and exception type of the public API.

Mirrors easier/core/utils.py:9-37: a ``logging`` logger named
``easier.init`` whose level comes from ``EASIER_LOG_LEVEL``, renamed
``Rank{r}`` by ``init``; ``EasierJitException`` for compile-time errors.
"""
import logging
import os

logger: logging.Logger = logging.getLogger("easier.init")
logger.setLevel(os.environ.get("EASIER_LOG_LEVEL", logging.INFO))
if not logger.handlers:
    _handler = logging.StreamHandler()
    _handler.setFormatter(logging.Formatter("%(asctime)s - %(name)s - %(levelname)s - %(message)s"))
    logger.addHandler(_handler)


def init_logger(rank: int) -> None:
    logger.name = f"Rank{rank}"


class EasierJitException(Exception):
    pass
