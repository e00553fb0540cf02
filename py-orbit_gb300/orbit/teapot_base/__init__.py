"""Python access to the TEAPOT maps (py/orbit/teapot_base/__init__.py)."""
import teapot_base as TPB

__all__ = ["TPB"]
