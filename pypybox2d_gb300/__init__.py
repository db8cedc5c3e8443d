"""pypybox2d_gb300 -- GB300 (sm_103a) implementation of pypybox2d's
World.step hot path behind the reference's World/Body/Fixture API."""
