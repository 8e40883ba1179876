"""CPU: argument checks of the field-count autotuner (no device needed)."""
import pytest


def test_autotune_fields_rejects_field_counts(built):
    """Batched domains hold 1 or a power of two >= 4 fields per node; the
    field-count autotuner refuses other candidates before touching a device."""
    from parallelfdtd_gb300.domain import autotune_fields
    for bad in ((3,), (6,), (12,)):
        with pytest.raises(ValueError):
            autotune_fields((16, 16, 16), lambda d: None, candidates=bad)
