"""Package logger (the counterpart of rubix/logger.py:10-61)."""

from __future__ import annotations

import logging


def get_logger(config=None) -> logging.Logger:
    """The "rubix_gb300" logger; ``config`` may set ``log_level`` and ``format``."""
    logger = logging.getLogger("rubix_gb300")
    if config:
        level = getattr(logging, str(config.get("log_level", "INFO")).upper(), logging.INFO)
        if logger.level != level:  # setLevel clears every logger's cache
            logger.setLevel(level)
        fmt = config.get("format")
        if fmt and not logger.handlers:
            h = logging.StreamHandler()
            h.setFormatter(logging.Formatter(fmt))
            logger.addHandler(h)
    return logger
