"""Host-side rules shared by the algorithms and the tile loop."""
