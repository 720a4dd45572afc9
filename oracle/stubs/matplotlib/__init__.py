"""No-op ``matplotlib`` stand-in so reference test modules import (test infrastructure only)."""
