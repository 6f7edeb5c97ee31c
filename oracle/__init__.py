"""CPU oracle for the splat render path (test infrastructure only)."""
