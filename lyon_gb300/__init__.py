"""GB300-native implementation of lyon's tessellation hot path (flatten, stroke, fill)."""
from .path import Path, PathBuilder, PathBatch, Verb
from .options import (FillOptions, FillRule, LineCap, LineJoin, Orientation, StrokeOptions)
