"""The ``xlumina`` import alias registers the reference's module names (no GPU)."""


def test_alias_registers_reference_module_names():
    import importlib

    import xlumina_gb300
    import xlumina_gb300.alias as alias
    alias.install()
    xl = importlib.import_module("xlumina")
    assert xl.um == 1 and xl.cm == 1e4 and xl.nm == 1e-3
    from xlumina.__init__ import cm  # noqa: F401  (the experiments' form)
    from xlumina import optical_elements, wave_optics
    from xlumina.vectorized_optics import VectorizedLight  # noqa: F401
    assert wave_optics is xlumina_gb300.wave_optics
    assert optical_elements.SLM is xlumina_gb300.optical_elements.SLM
