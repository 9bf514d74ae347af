"""Models of the reference's KPM tests (tests/test_kpm.py:7-14,138-143,168-173 and
cppcore/tests/test_kpm.cpp:7-17), built with the package's lattice restatement."""
from pybinding_gb300 import lattice as L


def graphene(kind, size):
    if kind == "pristine":
        return L.build_honeycomb(L.rectangle(size))
    if kind == "const_potential":
        return L.build_honeycomb(L.rectangle(size), onsite_modifiers=[L.constant_potential(0.5)])
    if kind == "magnetic_field":
        return L.build_honeycomb(L.rectangle(size), hopping_modifiers=[L.constant_magnetic_field(1e3)],
                                 is_complex=True)
    raise KeyError(kind)


LDOS_MODELS = {
    "graphene-pristine": ("pristine", 15),
    "graphene-pristine-oversized": ("pristine", 20),
    "graphene-const_potential": ("const_potential", 15),
    "graphene-magnetic_field": ("magnetic_field", 15),
}
DOS_MODELS = {"graphene-const_potential": ("const_potential", 25),
              "graphene-magnetic_field": ("magnetic_field", 25)}
COND_MODELS = {"graphene-const_potential": ("const_potential", 20),
               "graphene-magnetic_field": ("magnetic_field", 20)}


def cpp_fixture_model():
    """make_test_model(): 0.6 x 0.8 nm graphene + constant_potential(1), fixture lattice."""
    return L.build_honeycomb(L.rectangle(0.6, 0.8), onsite_modifiers=[L.constant_potential(1)],
                             min_neighbors=1, float_constants=True)


def cpp_fixture_model_plain():
    return L.build_honeycomb(L.rectangle(0.6, 0.8), min_neighbors=1, float_constants=True)
