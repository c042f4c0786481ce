"""CPU oracle for cannon_physics World.step -- test infrastructure only."""
