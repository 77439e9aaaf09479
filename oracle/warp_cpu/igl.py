"""Name-only stand-in for libigl (the third-party mesh library the
reference's utils/mesh.py imports at module level) -- TEST INFRASTRUCTURE
ONLY.  It is not installed here; none of its functions is called on the paths
the golden fixtures run (solid velocities of primitive bodies), so any use
raises AttributeError."""
