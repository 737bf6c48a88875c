"""distance3d_gb300 package (placeholder, filled below)."""
