"""Rounding and formatting helpers whose exact behaviour the grid build depends on."""
import decimal as d

import numpy as np


def round_value(value, decimalplaces=0):
    """Round like ``gprMax/utilities.py:116-136``.

    With ``decimalplaces == 0`` the value is rounded to the nearest integer with halves going
    down (``ROUND_HALF_DOWN``); this maps metres to cell indices. Otherwise it is rounded
    towards minus infinity at that many decimal places (``ROUND_FLOOR``); this is applied to
    the CFL time step so that it never exceeds the limit.
    """
    if isinstance(value, np.floating):
        value = float(value)
    if decimalplaces == 0:
        return int(d.Decimal(value).quantize(d.Decimal('1'), rounding=d.ROUND_HALF_DOWN))
    precision = '1.' + '0' * decimalplaces
    return float(d.Decimal(value).quantize(d.Decimal(precision), rounding=d.ROUND_FLOOR))


def round32(value):
    """Round up to the nearest multiple of 32."""
    return int(32 * np.ceil(float(value) / 32))


def human_size(size, a_kilobyte_is_1024_bytes=False):
    """Format a byte count for messages."""
    suffixes = {1000: ['KB', 'MB', 'GB', 'TB', 'PB'], 1024: ['KiB', 'MiB', 'GiB', 'TiB', 'PiB']}
    if size < 0:
        raise ValueError('Number must be non-negative.')
    multiple = 1024 if a_kilobyte_is_1024_bytes else 1000
    for suffix in suffixes[multiple]:
        size /= multiple
        if size < multiple:
            return '{:.3g}{}'.format(size, suffix)
    raise ValueError('Number is too large.')
