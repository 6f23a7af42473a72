"""The host device mirror's region and contact bookkeeping, on the case of the
reference's 2-D device test (tests/testDevice/testBasicDevice2D.hpp:36-155):
a 6 x 6 grid (maximum position 5 x 10, spacing 1 x 2) with four doping regions
and four contacts (ohmic, gate and ohmic on YMAX, ohmic on YMIN).

Expected values are the ones that test asserts; the engine reads exactly
these arrays through the device descriptor, so the test also checks them
there. Needs no GPU.
"""
import ctypes as C

import numpy as np
import pytest

from viennaemc_gb300.device import GATE, OHMIC, XMAX, XMIN, YMAX, YMIN, Device
from viennaemc_gb300.physics import Material


def _device():
    """testBasicDevice2D.hpp:41-51, 84-88."""
    silicon = Material(11.8, 2329.0, 1.45e16, 9040.0, 1.14)
    dev = Device(silicon, (5, 10), (1, 2))
    dev.addConstantDopingRegion((0, 0), (3, 6), 1e20)
    dev.addConstantDopingRegion((0, 6), (3, 10), 2e20)
    dev.addConstantDopingRegion((3, 0), (5, 6), 3e20)
    dev.addConstantDopingRegion((3, 6), (5, 10), 4e20)
    return dev


def _expected_region(x, y):
    """testBasicDevice2D.hpp:58-72: later regions overwrite shared nodes."""
    if x < 3 and y < 3:
        return 0, 1e20
    if x < 3:
        return 1, 2e20
    if y < 3:
        return 2, 3e20
    return 3, 4e20


def test_grid_extent_from_max_position_and_spacing():
    dev = _device()
    assert (dev.nx, dev.ny) == (6, 6)
    assert dev.getCellVolume() == pytest.approx(1 * 2 * 1e-6)


def test_doping_regions_of_the_reference_2d_device():
    dev = _device()
    assert dev.n_regions == 4
    for y in range(dev.ny):
        for x in range(dev.nx):
            idx, doping = _expected_region(x, y)
            assert dev.region[y * dev.nx + x] == idx, (x, y)
            assert dev.doping[y * dev.nx + x] == pytest.approx(doping, abs=1e-9)
    for r, doping in enumerate((1e20, 2e20, 3e20, 4e20)):
        assert dev.getDopingRegionDoping(r) == doping


def _add_contacts(dev):
    """testBasicDevice2D.hpp:81-88."""
    assert len(dev.contacts) == 0
    assert dev.addOhmicContact(YMAX, -2, (0,), (1,)) == 0
    assert dev.addGateContact(YMAX, 4, (2,), (3,), 1, 1, 1) == 1
    assert dev.addOhmicContact(YMAX, 2, (4,), (5,)) == 2
    assert dev.addOhmicContact(YMIN, 0, (0,), (5,)) == 3


def test_contacts_of_the_reference_2d_device():
    dev = _device()
    _add_contacts(dev)
    assert len(dev.contacts) == 4
    assert [c[0] for c in dev.contacts] == [OHMIC, GATE, OHMIC, OHMIC]
    assert [c[1] for c in dev.contacts] == [-2.0, 4.0, 2.0, 0.0]
    assert dev.contacts[1][2] == (1.0, 1.0, 1.0)
    # testBasicDevice2D.hpp:101-111: type at single surface coordinates,
    # artificial (no contact) boundary on XMIN and XMAX away from the corners
    assert dev.contacts[dev.bnd[YMIN][3]][0] == OHMIC
    assert dev.bnd[XMIN][3] == -1 and dev.bnd[XMAX][3] == -1
    assert dev.contacts[dev.bnd[YMAX][5]][0] == OHMIC
    assert dev.contacts[dev.bnd[YMAX][2]][0] == GATE
    assert dev.contacts[dev.bnd[YMAX][4]][0] == OHMIC


def _expected_contact(bp, c):
    """testBasicDevice2D.hpp:113-153, per surface coordinate: ohmic contacts
    also claim the corner nodes they share with the side boundaries; the gate
    does not."""
    if bp == YMIN:
        return 3
    if bp == YMAX:
        return 0 if c < 2 else (1 if c < 4 else 2)
    if c == 0:
        return 3
    if c == 5:
        return 0 if bp == XMIN else 2
    return -1


def test_boundary_contact_index_per_surface_node():
    dev = _device()
    _add_contacts(dev)
    volts = [-2.0, 4.0, 2.0, 0.0]
    for bp in (XMIN, XMAX, YMIN, YMAX):
        for c in range(len(dev.bnd[bp])):
            idx = int(dev.bnd[bp][c])
            assert idx == _expected_contact(bp, c), (bp, c)
            if bp in (YMIN, YMAX):
                assert volts[idx] == dev.contacts[idx][1]


def test_descriptor_carries_the_same_layout():
    dev = _device()
    _add_contacts(dev)
    d = dev.desc()
    assert (d.nx, d.ny, d.n_contacts) == (6, 6, 4)
    n = dev.nx * dev.ny
    region = np.ctypeslib.as_array(d.region, (n,))
    doping = np.ctypeslib.as_array(d.doping, (n,))
    for y in range(dev.ny):
        for x in range(dev.nx):
            idx, dop = _expected_region(x, y)
            assert region[y * dev.nx + x] == idx and doping[y * dev.nx + x] == dop
    for bp, length in ((XMIN, 6), (XMAX, 6), (YMIN, 6), (YMAX, 6)):
        got = np.ctypeslib.as_array(d.boundary_contact[bp], (length,))
        assert list(got) == [_expected_contact(bp, c) for c in range(length)]
    types = np.ctypeslib.as_array(d.contact_type, (4,))
    volts = np.ctypeslib.as_array(d.contact_voltage, (4,))
    params = np.ctypeslib.as_array(d.contact_param, (12,))
    assert list(types) == [OHMIC, GATE, OHMIC, OHMIC]
    assert list(volts) == [-2.0, 4.0, 2.0, 0.0]
    assert list(params[3:6]) == [1.0, 1.0, 1.0]
    assert isinstance(d.region, C.POINTER(C.c_int32))


def test_contact_outside_the_surface_is_rejected():
    dev = _device()
    with pytest.raises(ValueError, match="out of bounds"):
        dev.addOhmicContact(YMAX, 0, (0,), (7,))


def test_missing_doping_region_is_rejected():
    silicon = Material(11.8, 2329.0, 1.45e16, 9040.0, 1.14)
    dev = Device(silicon, (5, 10), (1, 2))
    dev.addConstantDopingRegion((0, 0), (5, 4), 1e20)
    with pytest.raises(ValueError, match="every discrete grid point"):
        dev.desc()
