"""Facet quadrature points of the reference facet rule, in cell reference
coordinates, as the reference computes them in float32 (its float32
least-squares facet maps evaluated in float32; element/element.py:1058-1066,
element/quadrature.py:321-410).  A float32 LAPACK solve cannot be restated
bit for bit, so the values are a table: written by tests/golden/make_golden.py
from the reference's own output, one float32 per entry (hex literal).
"""

POINTS = {
    ('triangle', 1): (
        ((float.fromhex('0x1.0000000000000p-1'), float.fromhex('0x1.0000000000000p-1'),),),
        ((float.fromhex('0x0.0p+0'), float.fromhex('0x1.0000000000000p-1'),),),
        ((float.fromhex('0x1.0000000000000p-1'), float.fromhex('0x0.0p+0'),),),
    ),
    ('triangle', 2): (
        ((float.fromhex('0x1.93cd380000000p-1'), float.fromhex('0x1.b0cb1a0000000p-3'),), (float.fromhex('0x1.b0cb200000000p-3'), float.fromhex('0x1.93cd380000000p-1'),),),
        ((float.fromhex('0x0.0p+0'), float.fromhex('0x1.b0cb1a0000000p-3'),), (float.fromhex('0x0.0p+0'), float.fromhex('0x1.93cd380000000p-1'),),),
        ((float.fromhex('0x1.b0cb1a0000000p-3'), float.fromhex('0x0.0p+0'),), (float.fromhex('0x1.93cd380000000p-1'), float.fromhex('0x0.0p+0'),),),
    ),
    ('triangle', 3): (
        ((float.fromhex('0x1.c64bf60000000p-1'), float.fromhex('0x1.cda0460000000p-4'),), (float.fromhex('0x1.0000000000000p-1'), float.fromhex('0x1.0000000000000p-1'),), (float.fromhex('0x1.cda0500000000p-4'), float.fromhex('0x1.c64bf60000000p-1'),),),
        ((float.fromhex('0x0.0p+0'), float.fromhex('0x1.cda0460000000p-4'),), (float.fromhex('0x0.0p+0'), float.fromhex('0x1.0000000000000p-1'),), (float.fromhex('0x0.0p+0'), float.fromhex('0x1.c64bf60000000p-1'),),),
        ((float.fromhex('0x1.cda0460000000p-4'), float.fromhex('0x0.0p+0'),), (float.fromhex('0x1.0000000000000p-1'), float.fromhex('0x0.0p+0'),), (float.fromhex('0x1.c64bf60000000p-1'), float.fromhex('0x0.0p+0'),),),
    ),
    ('triangle', 4): (
        ((float.fromhex('0x1.dc736c0000000p-1'), float.fromhex('0x1.1c64960000000p-4'),), (float.fromhex('0x1.5709000000000p-1'), float.fromhex('0x1.51ee000000000p-2'),), (float.fromhex('0x1.51ee000000000p-2'), float.fromhex('0x1.5708fe0000000p-1'),), (float.fromhex('0x1.1c64a00000000p-4'), float.fromhex('0x1.dc736c0000000p-1'),),),
        ((float.fromhex('0x0.0p+0'), float.fromhex('0x1.1c64960000000p-4'),), (float.fromhex('0x0.0p+0'), float.fromhex('0x1.51ee000000000p-2'),), (float.fromhex('0x0.0p+0'), float.fromhex('0x1.5708fe0000000p-1'),), (float.fromhex('0x0.0p+0'), float.fromhex('0x1.dc736c0000000p-1'),),),
        ((float.fromhex('0x1.1c64960000000p-4'), float.fromhex('0x0.0p+0'),), (float.fromhex('0x1.51ee000000000p-2'), float.fromhex('0x0.0p+0'),), (float.fromhex('0x1.5708fe0000000p-1'), float.fromhex('0x0.0p+0'),), (float.fromhex('0x1.dc736c0000000p-1'), float.fromhex('0x0.0p+0'),),),
    ),
    ('tetra', 1): (
        ((float.fromhex('0x1.5555500000000p-2'), float.fromhex('0x1.5555560000000p-2'), float.fromhex('0x1.5555560000000p-2'),),),
        ((float.fromhex('0x0.0p+0'), float.fromhex('0x1.5555560000000p-2'), float.fromhex('0x1.5555560000000p-2'),),),
        ((float.fromhex('0x1.5555560000000p-2'), float.fromhex('0x0.0p+0'), float.fromhex('0x1.5555560000000p-2'),),),
        ((float.fromhex('0x1.5555560000000p-2'), float.fromhex('0x1.5555560000000p-2'), float.fromhex('0x0.0p+0'),),),
    ),
    ('tetra', 2): (
        ((float.fromhex('0x1.5555540000000p-1'), float.fromhex('0x1.5555560000000p-3'), float.fromhex('0x1.55555a0000000p-3'),), (float.fromhex('0x1.55554c0000000p-3'), float.fromhex('0x1.5555540000000p-1'), float.fromhex('0x1.5555560000000p-3'),), (float.fromhex('0x1.5555500000000p-3'), float.fromhex('0x1.5555540000000p-3'), float.fromhex('0x1.5555560000000p-1'),),),
        ((float.fromhex('0x0.0p+0'), float.fromhex('0x1.5555560000000p-3'), float.fromhex('0x1.55555a0000000p-3'),), (float.fromhex('0x0.0p+0'), float.fromhex('0x1.5555540000000p-1'), float.fromhex('0x1.5555560000000p-3'),), (float.fromhex('0x0.0p+0'), float.fromhex('0x1.5555540000000p-3'), float.fromhex('0x1.5555560000000p-1'),),),
        ((float.fromhex('0x1.5555560000000p-3'), float.fromhex('0x0.0p+0'), float.fromhex('0x1.55555a0000000p-3'),), (float.fromhex('0x1.5555540000000p-1'), float.fromhex('0x0.0p+0'), float.fromhex('0x1.5555560000000p-3'),), (float.fromhex('0x1.5555540000000p-3'), float.fromhex('0x0.0p+0'), float.fromhex('0x1.5555560000000p-1'),),),
        ((float.fromhex('0x1.5555560000000p-3'), float.fromhex('0x1.55555a0000000p-3'), float.fromhex('0x0.0p+0'),), (float.fromhex('0x1.5555540000000p-1'), float.fromhex('0x1.5555560000000p-3'), float.fromhex('0x0.0p+0'),), (float.fromhex('0x1.5555540000000p-3'), float.fromhex('0x1.5555560000000p-1'), float.fromhex('0x0.0p+0'),),),
    ),
    ('tetra', 3): (
        ((float.fromhex('0x1.5555500000000p-2'), float.fromhex('0x1.5555560000000p-2'), float.fromhex('0x1.5555560000000p-2'),), (float.fromhex('0x1.9999900000000p-3'), float.fromhex('0x1.99999a0000000p-3'), float.fromhex('0x1.3333340000000p-1'),), (float.fromhex('0x1.9999900000000p-3'), float.fromhex('0x1.3333320000000p-1'), float.fromhex('0x1.99999c0000000p-3'),), (float.fromhex('0x1.3333300000000p-1'), float.fromhex('0x1.99999a0000000p-3'), float.fromhex('0x1.99999e0000000p-3'),),),
        ((float.fromhex('0x0.0p+0'), float.fromhex('0x1.5555560000000p-2'), float.fromhex('0x1.5555560000000p-2'),), (float.fromhex('0x0.0p+0'), float.fromhex('0x1.99999a0000000p-3'), float.fromhex('0x1.3333340000000p-1'),), (float.fromhex('0x0.0p+0'), float.fromhex('0x1.3333320000000p-1'), float.fromhex('0x1.99999c0000000p-3'),), (float.fromhex('0x0.0p+0'), float.fromhex('0x1.99999a0000000p-3'), float.fromhex('0x1.99999e0000000p-3'),),),
        ((float.fromhex('0x1.5555560000000p-2'), float.fromhex('0x0.0p+0'), float.fromhex('0x1.5555560000000p-2'),), (float.fromhex('0x1.99999a0000000p-3'), float.fromhex('0x0.0p+0'), float.fromhex('0x1.3333340000000p-1'),), (float.fromhex('0x1.3333320000000p-1'), float.fromhex('0x0.0p+0'), float.fromhex('0x1.99999c0000000p-3'),), (float.fromhex('0x1.99999a0000000p-3'), float.fromhex('0x0.0p+0'), float.fromhex('0x1.99999e0000000p-3'),),),
        ((float.fromhex('0x1.5555560000000p-2'), float.fromhex('0x1.5555560000000p-2'), float.fromhex('0x0.0p+0'),), (float.fromhex('0x1.99999a0000000p-3'), float.fromhex('0x1.3333340000000p-1'), float.fromhex('0x0.0p+0'),), (float.fromhex('0x1.3333320000000p-1'), float.fromhex('0x1.99999c0000000p-3'), float.fromhex('0x0.0p+0'),), (float.fromhex('0x1.99999a0000000p-3'), float.fromhex('0x1.99999e0000000p-3'), float.fromhex('0x0.0p+0'),),),
    ),
    ('tetra', 4): (
        ((float.fromhex('0x1.c8a6b60000000p-2'), float.fromhex('0x1.c8a6b80000000p-2'), float.fromhex('0x1.baca400000000p-4'),), (float.fromhex('0x1.7718900000000p-4'), float.fromhex('0x1.7718a00000000p-4'), float.fromhex('0x1.a239d80000000p-1'),), (float.fromhex('0x1.c8a6b60000000p-2'), float.fromhex('0x1.baca3c0000000p-4'), float.fromhex('0x1.c8a6b80000000p-2'),), (float.fromhex('0x1.7718a40000000p-4'), float.fromhex('0x1.a239d60000000p-1'), float.fromhex('0x1.7718a00000000p-4'),), (float.fromhex('0x1.baca380000000p-4'), float.fromhex('0x1.c8a6b80000000p-2'), float.fromhex('0x1.c8a6b80000000p-2'),), (float.fromhex('0x1.a239d40000000p-1'), float.fromhex('0x1.7718a20000000p-4'), float.fromhex('0x1.7718a80000000p-4'),),),
        ((float.fromhex('0x0.0p+0'), float.fromhex('0x1.c8a6b80000000p-2'), float.fromhex('0x1.baca400000000p-4'),), (float.fromhex('0x0.0p+0'), float.fromhex('0x1.7718a00000000p-4'), float.fromhex('0x1.a239d80000000p-1'),), (float.fromhex('0x0.0p+0'), float.fromhex('0x1.baca3c0000000p-4'), float.fromhex('0x1.c8a6b80000000p-2'),), (float.fromhex('0x0.0p+0'), float.fromhex('0x1.a239d60000000p-1'), float.fromhex('0x1.7718a00000000p-4'),), (float.fromhex('0x0.0p+0'), float.fromhex('0x1.c8a6b80000000p-2'), float.fromhex('0x1.c8a6b80000000p-2'),), (float.fromhex('0x0.0p+0'), float.fromhex('0x1.7718a20000000p-4'), float.fromhex('0x1.7718a80000000p-4'),),),
        ((float.fromhex('0x1.c8a6b80000000p-2'), float.fromhex('0x0.0p+0'), float.fromhex('0x1.baca400000000p-4'),), (float.fromhex('0x1.7718a00000000p-4'), float.fromhex('0x0.0p+0'), float.fromhex('0x1.a239d80000000p-1'),), (float.fromhex('0x1.baca3c0000000p-4'), float.fromhex('0x0.0p+0'), float.fromhex('0x1.c8a6b80000000p-2'),), (float.fromhex('0x1.a239d60000000p-1'), float.fromhex('0x0.0p+0'), float.fromhex('0x1.7718a00000000p-4'),), (float.fromhex('0x1.c8a6b80000000p-2'), float.fromhex('0x0.0p+0'), float.fromhex('0x1.c8a6b80000000p-2'),), (float.fromhex('0x1.7718a20000000p-4'), float.fromhex('0x0.0p+0'), float.fromhex('0x1.7718a80000000p-4'),),),
        ((float.fromhex('0x1.c8a6b80000000p-2'), float.fromhex('0x1.baca400000000p-4'), float.fromhex('0x0.0p+0'),), (float.fromhex('0x1.7718a00000000p-4'), float.fromhex('0x1.a239d80000000p-1'), float.fromhex('0x0.0p+0'),), (float.fromhex('0x1.baca3c0000000p-4'), float.fromhex('0x1.c8a6b80000000p-2'), float.fromhex('0x0.0p+0'),), (float.fromhex('0x1.a239d60000000p-1'), float.fromhex('0x1.7718a00000000p-4'), float.fromhex('0x0.0p+0'),), (float.fromhex('0x1.c8a6b80000000p-2'), float.fromhex('0x1.c8a6b80000000p-2'), float.fromhex('0x0.0p+0'),), (float.fromhex('0x1.7718a20000000p-4'), float.fromhex('0x1.7718a80000000p-4'), float.fromhex('0x0.0p+0'),),),
    ),
}
