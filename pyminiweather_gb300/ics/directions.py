"""Sweep directions, pyminiweather/ics/directions.py:4-6."""
from enum import Enum


class Directions(Enum):
    X = 0
    Z = 1
