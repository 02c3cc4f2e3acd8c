"""CPU oracle for the KMeans Lloyd path (test infrastructure only; see oracle.py)."""
