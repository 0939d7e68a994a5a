/* empty stand-in: nothing from this OpenCV header is used on the CPU path */
