"""Stub of ``torch_sla.distributed`` (imported by the reference's
distributed package at import time; never used for golden fixtures)."""


class DSparseTensor:
    pass
