"""Test and benchmark tooling beside the library, not part of it: seeded synthetic inputs shaped like the reference's
own channels and captures (synth). The library (lizard_gb300) never imports this package."""
