"""Empty stand-in so the reference's `from PIL import Image` imports (fixture generation only)."""
Image = None
