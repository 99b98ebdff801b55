"""One module per hot-path algorithm, ``algorithms/tile/<name>.py``, each
exposing the class that ``core.tile_loop._load_algorithm(name)`` instantiates
(the layout of the reference's algorithms/tile/ package)."""
